// Test infrastructure only: runs the UNMODIFIED reference DG patch solver
// (include/dg_helpers, header-only, compiled from its own sources by
// oracle/Makefile into oracle/_ref/) on a uniform tree and dumps the nodal
// DG state after initialisation and after every step, with the step sizes.
// The dumps become golden fixtures under tests/golden/ that pin the numpy
// restatement in oracle/dg_oracle.py and the CUDA DG path.  Nothing shipped
// links this file.
//
// Configuration: the reference's generated policy
// (include/config/generated_config.hpp: order 2, 2D, 4 variables per node,
// 4x4 cells per patch, one ghost cell, SSPRK2, advection with velocity 1).
// What the driver does, in the reference's own calls:
//   tree           the TreeBuilder's ndtree type (include/dg_helpers/
//                  tree_builder.hpp:399-403) with a small capacity (the
//                  builder itself allocates 500000 leaves), refined
//                  uniformly with reconstruct_tree;
//   initial state  GlobalConfig::compute_center and interpolate_initial_dofs
//                  per interior cell (tree_builder.hpp:407-466);
//   one step       DGSolver::advance_patches (include/dg_helpers/solver.hpp:
//                  159-232): halo exchange, begin_step, per stage a halo
//                  exchange and RHSEvaluator::evaluate + the SSPRK2 stage per
//                  patch, the CFL step from the last stage's largest
//                  eigenvalue, finish_step; the loop's step size rule
//                  dt = min(dt, dt_min) with dt = initial_dt at the start
//                  (solver.hpp:125-134);
//   re-mesh        with amr=<interval> > 0, DGSolver::apply_amr (solver.hpp:
//                  237-299) after each step from step 1 on, every interval
//                  steps: GradientAMRIndicator::compute_patch_decisions
//                  (include/dg_helpers/globals/amr_indicators.hpp:169-224) with
//                  thresholds rthr / cthr, reconstruct_tree with those
//                  decisions (the tree's DefaultAMRPolicy prolongation and
//                  restriction), halo exchange.
//   main loop      with end=<T> > 0 instead: DGSolver::run's loop (solver.hpp:
//                  109-151, without its VTK output) from time 0 while time < T:
//                  a step, dt = min(dt, dt_min), time += dt (the updated
//                  step), a re-mesh when the step count reaches the next
//                  re-mesh step, which then moves amr steps on; one dump of
//                  the final tree (step = steps run, dt = the next step size)
//                  and a line "steps remeshes cells leaves_max time next_dt"
//                  on stdout.
//   printer        with vtk=<file>: the final tree through the reference's DG
//                  printer (ndt::print::dg_tree_printer_2d, include/ndtree/
//                  print_dg_tree_v2.hpp; it writes under ./vtk_output, which
//                  it clears), the file then moved to <file>.
// Usage: ref_dg_driver level=<L> steps=<K> dt0=<initial dt> [amr=<interval>
//        rthr=<refine> cthr=<coarsen>] [end=<T>] [vtk=<file>] out=<file>
// Records: "DGS1" header, then per dump: step (u32), dt (f64), leaves
// (u64), ids (u64 x leaves), interior nodal values (f64 x leaves x 16 cells
// x 4 nodes x 4 variables, cells row-major with x fastest, nodes with the
// x-node index slowest as in the reference's tensor).
#include "config/generated_config.hpp"
#include "dg_helpers/globals/amr_indicators.hpp"
#include "dg_helpers/globals/global_config.hpp"
#include "dg_helpers/rhs.hpp"
#include "dg_helpers/time_integration/time_integration.hpp"
#include "dg_helpers/tree_builder.hpp"
#include "ndtree/print_dg_tree_v2.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

namespace
{
// The generated policy fixes the equation to advection; built with
// -DDG_EULER the driver runs the same configuration with the reference's DG
// Euler equations (include/dg_helpers/equations/euler.hpp) instead.
#ifdef DG_EULER
struct EulerPolicy : amr::config::GlobalConfigPolicy
{
    static constexpr amr::config::EquationType equation = amr::config::EquationType::Euler;
};
using policy_t = EulerPolicy;
#else
using policy_t = amr::config::GlobalConfigPolicy;
#endif
using global_t          = amr::global::GlobalConfig<policy_t>;
using rhs_t             = amr::rhs::RHSEvaluator<global_t, policy_t>;
using builder_t         = amr::dg_tree::TreeBuilder<global_t, policy_t>;
using S1                = builder_t::S1;
using S2                = builder_t::S2;
using S3                = builder_t::S3;
using S4                = builder_t::S4;
using tree_t            = builder_t::tree_t;
using patch_layout_t    = builder_t::patch_layout_t;
using patch_index_t     = builder_t::patch_index_t;
using patch_container_t = amr::containers::static_tensor<S1::type, patch_layout_t::padded_layout_t>;
using integrator_t =
    amr::time_integration::TimeIntegratorTraits<policy_t::integrator, patch_container_t>::type;

long arg(int argc, char** argv, const char* key, long dflt)
{
    const std::size_t n = std::strlen(key);
    for (int i = 1; i < argc; ++i)
        if (std::strncmp(argv[i], key, n) == 0 && argv[i][n] == '=') return std::strtol(argv[i] + n + 1, nullptr, 10);
    return dflt;
}
double argf(int argc, char** argv, const char* key, double dflt)
{
    const std::size_t n = std::strlen(key);
    for (int i = 1; i < argc; ++i)
        if (std::strncmp(argv[i], key, n) == 0 && argv[i][n] == '=') return std::strtod(argv[i] + n + 1, nullptr);
    return dflt;
}
std::string args(int argc, char** argv, const char* key, const char* dflt)
{
    const std::size_t n = std::strlen(key);
    for (int i = 1; i < argc; ++i)
        if (std::strncmp(argv[i], key, n) == 0 && argv[i][n] == '=') return argv[i] + n + 1;
    return dflt;
}

// interior nodal values of every leaf, in leaf order
void dump(std::FILE* f, tree_t& tree, std::uint32_t step, double dt)
{
    std::fwrite(&step, sizeof step, 1, f);
    std::fwrite(&dt, sizeof dt, 1, f);
    const std::uint64_t P = tree.size();
    std::fwrite(&P, sizeof P, 1, f);
    for (std::size_t i = 0; i < P; ++i)
    {
        const std::uint64_t id = tree.get_node_index_at(i).id();
        std::fwrite(&id, sizeof id, 1, f);
    }
    for (std::size_t i = 0; i < P; ++i)
    {
        auto& dof = tree.template get_patch<S1>(i);
        for (std::size_t lin = 0; lin < patch_layout_t::flat_size(); ++lin)
        {
            if (amr::ndt::utils::patches::is_halo_cell<patch_layout_t>(lin)) continue;
            const auto& cell = dof[lin];
            for (std::size_t k = 0; k < S1::type::elements(); ++k)
                for (std::size_t v = 0; v < policy_t::DOFs; ++v)
                {
                    const double x = cell[k][v];
                    std::fwrite(&x, sizeof x, 1, f);
                }
        }
    }
}

// one DGSolver step (advance_patches), re-mesh left out
void step(tree_t& tree, double dt, double& dt_min)
{
    const int                 n_stages = integrator_t::num_stages();
    std::vector<integrator_t> integ(tree.size());
    tree.halo_exchange_update();
    for (std::size_t i = 0; i < tree.size(); ++i) integ[i].begin_step(tree.template get_patch<S1>(i).data());
    for (int s = 0; s < n_stages; ++s)
    {
        tree.halo_exchange_update();
        for (std::size_t i = 0; i < tree.size(); ++i)
        {
            auto&        dof     = tree.template get_patch<S1>(i);
            auto&        flux    = tree.template get_patch<S2>(i);
            const double edge    = global_t::cell_edge(tree.get_node_index_at(i));
            const double volume  = global_t::cell_volume(edge);
            const double surface = global_t::cell_area(edge);
            const double inv_jac = 1.0 / edge;
            double       lam     = -std::numeric_limits<double>::infinity();
            auto         res = [&](patch_container_t& upd, const patch_container_t& cur, double) {
                rhs_t::evaluate(cur, flux.data(), upd, dt, volume, surface, lam, inv_jac);
            };
            integ[i].compute_stage(s, res, dof.data(), 0.0, dt);
            dof.data() = integ[i].stage_result(s, dof.data());
            if (s == n_stages - 1 && lam > 0.0)
            {
                const double scale = 1.0 / (std::pow(policy_t::Order, policy_t::Dim) + 1.0);
                dt_min             = std::min(dt_min, scale * amr::config::CourantNumber * edge / lam);
            }
        }
    }
    for (std::size_t i = 0; i < tree.size(); ++i) integ[i].finish_step(tree.template get_patch<S1>(i).data());
}
} // namespace

int main(int argc, char** argv)
{
    const int         level = static_cast<int>(arg(argc, argv, "level", 2));
    const int         steps = static_cast<int>(arg(argc, argv, "steps", 3));
    double            dt    = argf(argc, argv, "dt0", 0.01);
    const std::string out   = args(argc, argv, "out", "dg.bin");
    std::FILE*        f     = std::fopen(out.c_str(), "wb");
    if (!f)
    {
        std::perror(out.c_str());
        return 2;
    }
    tree_t tree{ static_cast<std::size_t>(arg(argc, argv, "capacity", (1L << (2 * level)) + 64)) };
    auto   refine_all = [](const patch_index_t&) { return tree_t::refine_status_t::Refine; };
    for (int l = 0; l < level; ++l) tree.reconstruct_tree(refine_all);
    for (std::size_t i = 0; i < tree.size(); ++i)
    {
        auto&        dof    = tree.template get_patch<S1>(i);
        auto&        flux   = tree.template get_patch<S2>(i);
        auto&        center = tree.template get_patch<S3>(i);
        auto&        size   = tree.template get_patch<S4>(i);
        const auto   pid    = tree.get_node_index_at(i);
        auto [pc, pl]       = patch_index_t::decode(pid.id());
        const double cell   = (1.0 / static_cast<double>(1u << pl)) / static_cast<double>(policy_t::PatchSize);
        for (std::size_t lin = 0; lin != patch_layout_t::flat_size(); ++lin)
        {
            if (amr::ndt::utils::patches::is_halo_cell<patch_layout_t>(lin)) continue;
            const auto c = global_t::compute_center(pid, global_t::rm_halo(global_t::lin_to_local(lin)));
            center[lin]  = c;
            dof[lin]     = global_t::interpolate_initial_dofs(c, cell);
            flux[lin]    = typename std::remove_reference_t<decltype(flux)>::value_type{};
            size[lin]    = typename std::remove_reference_t<decltype(size)>::value_type{};
        }
    }
    tree.halo_exchange_update();
    std::fwrite("DGS1", 1, 4, f);
    dump(f, tree, 0, 0.0);
    const int                   amr_every = static_cast<int>(arg(argc, argv, "amr", 0));
    amr::global::AMRThresholds  thr{ argf(argc, argv, "rthr", 0.05), argf(argc, argv, "cthr", 0.01) };
    int                         next_amr = 0;
    using indicator_t = amr::global::GradientAMRIndicator<global_t, policy_t>;
    using status_t    = tree_t::refine_status_t;
    auto remesh       = [&]() {
        const auto decisions = indicator_t::template compute_patch_decisions<tree_t, S1>(tree, thr);
        std::unordered_map<patch_index_t, status_t> by_id;
        for (std::size_t i = 0; i < decisions.size(); ++i) by_id[tree.get_node_index_at(i)] = decisions[i];
        tree.reconstruct_tree([&by_id](const patch_index_t& pid) -> status_t {
            auto it = by_id.find(pid);
            return it != by_id.end() ? it->second : status_t::Stable;
        });
        tree.halo_exchange_update();
    };
    const std::string vtk = args(argc, argv, "vtk", "");
    auto print_vtk        = [&]() {
        if (vtk.empty()) return;
        ::ndt::print::dg_tree_printer_2d<global_t, policy_t> printer("dg");
        printer.template print<S1>(tree, "_final.vtk");
        for (const auto& e : std::filesystem::directory_iterator("vtk_output"))
        {
            std::filesystem::copy_file(e.path(), vtk, std::filesystem::copy_options::overwrite_existing);
            std::filesystem::remove(e.path());
        }
    };
    const double end = argf(argc, argv, "end", 0.0);
    if (end > 0.0)
    {
        double        time = 0.0;
        std::uint64_t k = 0, remeshes = 0, cells = 0, leaves_max = tree.size();
        while (time < end)
        {
            double dt_min = dt;
            step(tree, dt, dt_min);
            dt = std::min(dt, dt_min);
            cells += tree.size() * 16;
            time += dt;
            ++k;
            if (static_cast<long>(k) >= next_amr)
            {
                remesh();
                ++remeshes;
                next_amr   = static_cast<int>(k) + amr_every;
                leaves_max = std::max<std::uint64_t>(leaves_max, tree.size());
            }
        }
        dump(f, tree, static_cast<std::uint32_t>(k), dt);
        std::fclose(f);
        print_vtk();
        std::printf("%llu %llu %llu %llu %.17g %.17g\n", static_cast<unsigned long long>(k),
                    static_cast<unsigned long long>(remeshes), static_cast<unsigned long long>(cells),
                    static_cast<unsigned long long>(leaves_max), time, dt);
        return 0;
    }
    for (int k = 1; k <= steps; ++k)
    {
        double dt_min = dt;
        step(tree, dt, dt_min);
        const double used = dt;
        dt                = std::min(dt, dt_min);
        if (amr_every > 0 && k >= next_amr)
        {
            remesh();
            next_amr = k + amr_every;
        }
        dump(f, tree, static_cast<std::uint32_t>(k), used);
    }
    std::fclose(f);
    print_vtk();
    return 0;
}
