// Compressible Euler plug-in with the static interface of gpu-amr's
// EulerPhysics<DIM> (include/solver/EulerPhysics.hpp:17-185).  The Rusanov
// update and the CFL step run in the CUDA kernels (amr_tree_euler_advance);
// this type supplies NVAR, the field tags and the primitive -> conservative
// map used by amr_solver::initialize, with the reference's operation order.
#pragma once

#include "containers/static_vector.hpp"
#include "solver/cell_types.hpp"

#include <tuple>
#include <type_traits>

template <int DIM>
class EulerPhysics
{
public:
    static constexpr int NVAR = DIM + 2;
    using FieldTags           = std::conditional_t<
        DIM == 2, std::tuple<amr::cell::Rho, amr::cell::Rhou, amr::cell::Rhov, amr::cell::E2D>,
        std::tuple<amr::cell::Rho, amr::cell::Rhou, amr::cell::Rhov, amr::cell::Rhow, amr::cell::E3D>>;

    // [rho, u_d..., p] -> [rho, rho u_d..., p / (gamma - 1) + 0.5 rho |u|^2]
    static void primitiveToConservative(const amr::containers::static_vector<double, NVAR>& prim,
                                        amr::containers::static_vector<double, NVAR>& cons, double gamma)
    {
        const double rho = prim[0];
        double       v2  = 0.0;
        cons[0]          = rho;
        for (int d = 0; d < DIM; ++d) {
            const double u = prim[1 + d];
            cons[1 + d]    = rho * u;
            v2 += u * u;
        }
        cons[DIM + 1] = prim[DIM + 1] / (gamma - 1.0) + 0.5 * rho * v2;
    }

    static constexpr int getNumVars() { return NVAR; }
};

using EulerPhysics2D = EulerPhysics<2>;
using EulerPhysics3D = EulerPhysics<3>;

namespace Direction
{
constexpr int X = 0;
constexpr int Y = 1;
constexpr int Z = 2;
} // namespace Direction
