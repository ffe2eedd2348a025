// gpu-amr's DG solver (include/dg_helpers/solver.hpp: SimulationParams,
// DGSolver<Policy>) on the GB300 device tree: the same names, parameters and
// loop, with every step, re-mesh and output on the device through the C ABI
// (amr_tree_dg_advance, amr_tree_dg_remesh, amr_tree_dg_write_vtk).  The
// tree is built like the reference's TreeBuilder (tree_builder.hpp:407-466):
// uniform refinement to the initial level, then the equation's initial
// values at each cell's Gauss-Legendre nodes (GlobalConfig::
// interpolate_initial_dofs), computed here on the host with the reference's
// arithmetic and uploaded.  Compile with ISO C++ (-std=c++20: no
// floating-point contraction) for initial values identical to the
// reference's.
#pragma once

#include "amr_gb300.h"
#include "config/generated_config.hpp"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <vector>

namespace amr::global
{
// Gradient indicator thresholds (dg_helpers/globals/amr_indicators.hpp:19-23)
struct AMRThresholds
{
    double refine_threshold  = 0.5;
    double coarsen_threshold = 0.05;
};
} // namespace amr::global

namespace amr::solver
{

struct SimulationParams
{
    double initial_dt    = 0.01;
    double plot_interval = 0.01;
    int    initial_level = 4;
    int    amr_interval  = 200;

    amr::global::AMRThresholds amr_thresholds = { .refine_threshold = 0.05, .coarsen_threshold = 0.01 };
};

namespace detail
{
inline void dg_check(amr_status s)
{
    if (s != AMR_OK) throw std::runtime_error(amr_last_error());
}
} // namespace detail

template <typename Policy>
struct DGSolver
{
    static_assert(Policy::Order == 2 && Policy::Dim == 2 && Policy::DOFs == 4 && Policy::PatchSize == 4 &&
                      Policy::HaloWidth == 1,
                  "the device DG path is built for order 2, 2D, 4 variables, 4x4 cells, one ghost cell");
    static_assert(Policy::integrator == amr::config::TimeIntegratorType::SSPRK2, "SSPRK2");
    static_assert(amr::config::CourantNumber == 0.5, "Courant number 0.5");

    static constexpr std::size_t capacity = 500000; // the TreeBuilder's tree (tree_builder.hpp:405)

    SimulationParams params;

    explicit DGSolver(SimulationParams p = {}) : params{ p }
    {
        amr_tree_desc d{};
        d.geom.rank  = 2;
        d.geom.n     = 4;
        d.geom.halo  = 1;
        d.geom.depth = static_cast<int32_t>(Policy::MaxDepth);
        for (int a = 0; a < 3; ++a) d.geom.lengths[a] = 1.0;
        d.capacity = capacity;
        d.dtype    = AMR_F64;
        d.fields   = 16;
        detail::dg_check(amr_tree_create(&d, &m_tree));
        if constexpr (Policy::equation == amr::config::EquationType::Euler)
            detail::dg_check(amr_tree_dg_set_equation(m_tree, AMR_DG_EULER));
        detail::dg_check(amr_tree_refine_uniform(m_tree, p.initial_level));
        upload_initial_values();
    }
    ~DGSolver()
    {
        if (m_tree) amr_tree_destroy(m_tree);
    }
    DGSolver(DGSolver const&)            = delete;
    DGSolver& operator=(DGSolver const&) = delete;

    amr_tree* tree() const { return m_tree; }

    // processed cells (leaves x 16 per step) and wall seconds of the last run()
    std::size_t processed_cells() const { return m_processed; }
    double      seconds() const { return m_seconds; }

private:
    amr_tree*   m_tree      = nullptr;
    std::size_t m_processed = 0;
    double      m_seconds   = 0.0;

    // get_initial_values of the equation at a node (advection.hpp:69-86,
    // euler.hpp:227-253), variables in the tree's order
    static void initial_values(double x, double y, double* v)
    {
        if constexpr (Policy::equation == amr::config::EquationType::Euler) {
            const double r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5);
            const double p  = std::exp(-100.0 * r2) + 1.0;
            v[0] = 0.0;
            v[1] = 0.0;
            v[2] = 1.0;
            v[3] = p / (1.4 - 1.0);
        } else {
            const double pi = 3.14159265358979323846;
            v[0]            = std::sin(2.0 * pi * (x + y - 2.0 * 0.0));
            v[1]            = std::sin(2.0 * pi * (y - 0.0));
            v[2]            = 1.0;
            v[3]            = 1.0;
        }
    }

    void upload_initial_values()
    {
        std::size_t P = 0;
        detail::dg_check(amr_tree_size(m_tree, &P));
        std::vector<uint64_t> ids(P);
        detail::dg_check(amr_tree_get_ids(m_tree, ids.data(), P));
        const std::vector<double> state = initial_state(ids);
        detail::dg_check(amr_tree_upload_state(m_tree, state.data(), P));
    }

public:
    // TreeBuilder's initial state for the leaves `ids` (Morton ids of this
    // policy's depth): per interior cell, the centre (patch corner + (local +
    // 0.5) x cell edge) and the values at the nodes centre + (point - 1/2) x
    // edge; fields x leaves x 6 x 6, ghosts zero
    static std::vector<double> initial_state(const std::vector<uint64_t>& ids)
    {
        const std::size_t   P = ids.size();
        std::vector<double> state(16 * P * 36, 0.0);
        const double        pts[2] = { 0.5 + 0.5 * -0.5773502691896257, 0.5 + 0.5 * 0.5773502691896257 };
        const double        unit   = 1.0 / static_cast<double>(1u << Policy::MaxDepth);
        for (std::size_t i = 0; i < P; ++i) {
            const uint64_t m = ids[i] >> 6;
            uint32_t       cx = 0, cy = 0;
            for (unsigned b = 0; b < Policy::MaxDepth; ++b) {
                cx |= static_cast<uint32_t>((m >> (2 * b)) & 1u) << b;
                cy |= static_cast<uint32_t>((m >> (2 * b + 1)) & 1u) << b;
            }
            const int    level = static_cast<int>(ids[i] & 63u);
            const double edge  = (1.0 / static_cast<double>(1u << level)) / 4.0;
            for (int ly = 0; ly < 4; ++ly)
                for (int lx = 0; lx < 4; ++lx) {
                    const double ccx = static_cast<double>(cx) * unit + (static_cast<double>(lx) + 0.5) * edge;
                    const double ccy = static_cast<double>(cy) * unit + (static_cast<double>(ly) + 0.5) * edge;
                    for (int ix = 0; ix < 2; ++ix)
                        for (int iy = 0; iy < 2; ++iy) {
                            double v[4];
                            initial_values(ccx + (pts[ix] - 0.5) * edge, ccy + (pts[iy] - 0.5) * edge, v);
                            for (int var = 0; var < 4; ++var)
                                state[((((ix * 2 + iy) * 4 + var) * P) + i) * 36 + (ly + 1) * 6 + lx + 1] = v[var];
                        }
                }
        }
        return state;
    }

    // DGSolver::run (solver.hpp:109-151): output at time 0, then steps while
    // time < EndTime: the step (dt = min(dt, dt_min), time += dt), a
    // re-mesh when the step count reaches the next re-mesh step
    // (apply_amr, solver.hpp:249-310), output when time reaches the next
    // plot time.  The printer's folder ./vtk_output is cleared first, as
    // the reference's printer does on construction.
    void run()
    {
        const std::filesystem::path dir("vtk_output");
        if (std::filesystem::exists(dir)) std::filesystem::remove_all(dir);
        std::filesystem::create_directory(dir);

        double time           = 0.0;
        double dt             = params.initial_dt;
        int    timestep       = 0;
        double next_plot_time = 0.01;
        int    next_amr_step  = 0;
        write_output(timestep);

        m_processed      = 0;
        const auto start = std::chrono::steady_clock::now();
        while (time < Policy::EndTime) {
            std::size_t P = 0;
            detail::dg_check(amr_tree_size(m_tree, &P));
            detail::dg_check(amr_tree_dg_advance(m_tree, 1, &dt, &time));
            m_processed += P * 16;
            ++timestep;
            if (timestep >= next_amr_step) {
                detail::dg_check(amr_tree_dg_remesh(m_tree, params.amr_thresholds.refine_threshold,
                                                    params.amr_thresholds.coarsen_threshold, nullptr));
                next_amr_step = timestep + params.amr_interval;
            }
            if (time >= next_plot_time) {
                write_output(timestep);
                next_plot_time += params.plot_interval;
            }
        }
        detail::dg_check(amr_tree_synchronize(m_tree));
        m_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    }

private:
    // write_output (solver.hpp:315-320) with the printer's file name
    // (print_dg_tree_v2.hpp:145-163)
    void write_output(int timestep)
    {
        std::string name = "vtk_output/DG_";
        name += Policy::equation == amr::config::EquationType::Euler ? "Euler" : "Advection";
        name += "_ord" + std::to_string(Policy::Order) + "_SSPRK2_t" + std::to_string(timestep) + ".vtk";
        detail::dg_check(amr_tree_dg_write_vtk(m_tree, name.c_str()));
    }
};

} // namespace amr::solver
