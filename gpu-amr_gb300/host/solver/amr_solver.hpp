// gpu-amr's amr_solver<TreeT, GeometryT, EquationT, DIM>
// (include/solver/amr_solver.hpp:28-544) on the GB300 device-resident tree:
// initialize() evaluates the initial condition on the host like the
// reference (amr_solver.hpp:105-145); advance_batch_async /
// finish_advance_batch run forward-Euler Rusanov steps on the GPU with the CFL
// step clamped to the remaining time: linear advection (NVAR = 1, dt = cfl *
// min dx/|v|) or compressible Euler (NVAR = DIM + 2, EulerPhysics, dt = cfl *
// min dx/(|u| + a), amr_tree_euler_advance).
#pragma once

#include "ndtree/ndtree.hpp"
#include "containers/static_vector.hpp"

#include <array>
#include <functional>
#include <limits>

template <typename TreeT, typename GeometryT, typename EquationT, int DIM>
class amr_solver
{
public:
    using tree_t          = TreeT;
    using patch_layout_t  = typename tree_t::patch_layout_t;
    using patch_index_t   = typename tree_t::patch_index_t;
    using padded_layout_t = typename patch_layout_t::padded_layout_t;
    static constexpr auto NVAR = EquationT::NVAR;
    using arithmetic_t         = double;
    static_assert(DIM == 2 || DIM == 3, "Error: Wrong dimension");
    static constexpr bool euler = NVAR == DIM + 2;
    static_assert(NVAR == 1 || euler, "advection (one field) or Euler (DIM + 2 fields)");
    static_assert(NVAR == static_cast<int>(tree_t::n_fields), "the cell carries the equation's fields");

    amr_solver(std::size_t capacity, arithmetic_t gamma_ = 1.4, arithmetic_t cfl_ = 0.1)
        : m_tree(capacity, domain_lengths()), m_gamma(gamma_), m_cfl(cfl_)
    {
        if constexpr (!euler)
            for (int a = 0; a < 3; ++a) m_velocity[a] = EquationT::Velocity[a];
    }

    auto get_tree() -> TreeT& { return m_tree; }
    auto get_gamma() const noexcept -> arithmetic_t { return m_gamma; }
    auto get_cfl() const noexcept -> arithmetic_t { return m_cfl; }
    void set_velocity(std::array<double, 3> const& v) { m_velocity = v; }

    void initialize(auto&& init_func)
    {
        for (std::size_t p = 0; p < m_tree.size(); ++p) {
            const auto id = m_tree.get_node_index_at(p);
            const auto cs = GeometryT::cell_sizes(id);
            for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li) {
                if (amr::ndt::utils::patches::is_halo_cell<patch_layout_t>(
                        static_cast<typename patch_layout_t::index_t>(li)))
                    continue;
                const auto origin = GeometryT::cell_coord(id, static_cast<typename padded_layout_t::index_t>(li));
                std::array<arithmetic_t, DIM> coords;
                for (int d = 0; d < DIM; ++d) coords[d] = origin[d] + 0.5 * cs[d];
                const auto prim = std::invoke(init_func, coords);
                amr::containers::static_vector<arithmetic_t, NVAR> cons;
                EquationT::primitiveToConservative(prim, cons, m_gamma);
                for (int f = 0; f < NVAR; ++f)
                    m_tree.get_field_patch(static_cast<std::size_t>(f), p)[static_cast<typename patch_layout_t::index_t>(li)] =
                        cons[f];
            }
        }
    }

    auto advance() -> arithmetic_t
    {
        advance_batch_async(1);
        return finish_advance_batch();
    }

    void advance_batch_async(std::size_t step_count,
                             arithmetic_t remaining_time = std::numeric_limits<arithmetic_t>::max())
    {
        if constexpr (euler)
            amr::gb300::check(amr_tree_euler_advance(m_tree.handle(), step_count, m_gamma, m_cfl, remaining_time));
        else
            amr::gb300::check(amr_tree_advance(m_tree.handle(), step_count, m_velocity.data(), m_cfl, remaining_time));
    }

    auto finish_advance_batch(std::size_t* executed_step_count = nullptr) -> arithmetic_t
    {
        double      sum = 0.0;
        std::size_t ex  = 0;
        amr::gb300::check(amr_tree_finish_advance(m_tree.handle(), &sum, &ex));
        if (executed_step_count) *executed_step_count = ex;
        return sum;
    }

    // The reference benchmark loop on the device (amr_tree_run): `steps`
    // steps, re-mesh with the criterion every `interval` steps.
    auto run(std::size_t steps, std::size_t interval, amr::gb300::gradient_criterion const& c,
             arithmetic_t remaining_time = std::numeric_limits<arithmetic_t>::max()) -> amr_cycle_stats
    {
        static_assert(!euler, "Euler: run_euler");
        amr_cycle_params prm{};
        prm.steps           = steps;
        prm.remesh_interval = interval;
        for (int a = 0; a < 3; ++a) prm.velocity[a] = m_velocity[a];
        prm.cfl               = m_cfl;
        prm.remaining_time    = remaining_time;
        prm.criterion         = 1;
        prm.min_level         = c.min_level;
        prm.max_level         = c.max_level;
        prm.refine_threshold  = c.refine_threshold;
        prm.coarsen_threshold = c.coarsen_threshold;
        amr_cycle_stats st{};
        amr::gb300::check(amr_tree_run(m_tree.handle(), &prm, &st));
        return st;
    }

    // The Euler benchmark loop on the device (amr_tree_euler_run): advance
    // `interval` steps with the time left, max-Rho flags, re-mesh, until
    // `steps` steps ran or the simulated time reaches end_time.
    auto run_euler(std::size_t steps, std::size_t interval, double end_time,
                   amr::gb300::max_value_criterion const& c) -> amr_cycle_stats
    {
        static_assert(euler, "the equation is not Euler");
        amr_euler_params prm{};
        prm.steps             = steps;
        prm.remesh_interval   = interval;
        prm.gamma             = m_gamma;
        prm.cfl               = m_cfl;
        prm.end_time          = end_time;
        prm.refine_threshold  = c.refine_threshold;
        prm.coarsen_threshold = c.coarsen_threshold;
        prm.min_level         = c.min_level;
        prm.max_level         = c.max_level;
        amr_cycle_stats st{};
        amr::gb300::check(amr_tree_euler_run(m_tree.handle(), &prm, &st));
        return st;
    }

private:
    static auto domain_lengths() -> std::array<double, 3>
    {
        std::array<double, 3> l{ 1.0, 1.0, 1.0 };
        for (int d = 0; d < DIM; ++d) l[d] = GeometryT::domain_length(d);
        return l;
    }

    TreeT                 m_tree;
    arithmetic_t          m_gamma;
    arithmetic_t          m_cfl;
    std::array<double, 3> m_velocity{};
};

template <typename TreeT, typename GeometryT, typename EquationT>
using amr_solver_2d = amr_solver<TreeT, GeometryT, EquationT, 2>;
template <typename TreeT, typename GeometryT, typename EquationT>
using amr_solver_3d = amr_solver<TreeT, GeometryT, EquationT, 3>;
