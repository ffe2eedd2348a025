// The reference's own solver tests (tests/advection_equation_amr.t.cpp), the
// type definitions and test bodies kept as they are, compiled against the
// GB300 drop-in headers (gpu-amr_gb300/host) and linked with libamr_gb300.
// GoogleTest is replaced by a minimal EXPECT_NEAR.  A second mode runs the
// reference benchmark loop (bench_fvm_solver_integration_active_amr.b.cpp:
// 220-250) on the config-2 workload and prints the final tree and state for
// comparison with the oracle; a third runs the Euler benchmark's set-up and
// loop (bench_fvm_solver_integration.b.cpp:34-250: EulerCell2D, acoustic
// pulse, host max-Rho criterion) on 8x8 patches.
#include "containers/static_layout.hpp"
#include "containers/static_shape.hpp"
#include "containers/static_vector.hpp"
#include "morton/morton_id.hpp"
#include "ndtree/intergrid_operator.hpp"
#include "ndtree/ndtree.hpp"
#include "ndtree/patch_layout.hpp"
#include "ndtree/vtk_print.hpp"
#include "solver/AdvectionPhysics.hpp"
#include "solver/EulerPhysics.hpp"
#include "solver/adjoint.hpp"
#include "solver/amr_solver.hpp"
#include "solver/cell_types.hpp"
#include "solver/physics_system.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

static int g_failures = 0;
#define EXPECT_NEAR(a, b, tol)                                                                          \
    do {                                                                                                \
        if (!(std::abs((a) - (b)) <= (tol))) {                                                          \
            std::cout << "FAIL " << __LINE__ << ": " << (a) << " vs " << (b) << " tol " << (tol) << "\n"; \
            ++g_failures;                                                                               \
        }                                                                                               \
    } while (0)

template <int Dim, std::size_t PatchDim>
struct AdvectionTestConfig
{
    static constexpr int DIM = Dim;
    using shape_t            = amr::containers::static_shape<PatchDim, PatchDim>;
    using layout_t           = amr::containers::static_layout<shape_t>;
    using patch_index_t      = amr::ndt::morton::morton_id<7u, 2u>;
    using patch_layout_t     = amr::ndt::patches::patch_layout<layout_t, 2>;
    using equation_t         = AdvectionPhysics<Dim>;
    using cell_t             = amr::cell::AdvectionCell;
    using intergrid_operator_t = amr::ndt::intergrid_operator::linear_interpolator<patch_layout_t>;
    using tree_t = amr::ndt::tree::ndtree<cell_t, patch_index_t, patch_layout_t, intergrid_operator_t>;
    static constexpr std::array<double, Dim> domain_lengths = { 1.0, 1.0 };
    using geometry_t = amr::ndt::solver::physics_system<patch_index_t, patch_layout_t, domain_lengths>;
};

template <typename Config>
void find_peak(typename Config::tree_t& tree, std::array<double, 2>& actual_pos)
{
    double max_val = -1.0;
    for (std::size_t p_idx = 0; p_idx < tree.size(); ++p_idx) {
        auto        patch_id = tree.get_node_index_at(p_idx);
        auto const& patch    = tree.template get_patch<amr::cell::Scalar>(p_idx);
        for (std::size_t l_idx = 0; l_idx < Config::patch_layout_t::flat_size(); ++l_idx) {
            if (amr::ndt::utils::patches::is_halo_cell<typename Config::patch_layout_t>(l_idx)) continue;
            if (patch[l_idx] > max_val) {
                max_val    = patch[l_idx];
                auto coord = Config::geometry_t::cell_coord(patch_id, l_idx);
                auto size  = Config::geometry_t::cell_sizes(patch_id);
                for (int d = 0; d < Config::DIM; ++d) actual_pos[d] = coord[d] + 0.5 * size[d];
            }
        }
    }
}

template <typename Config>
void PulseCenterMovement()
{
    amr_solver<typename Config::tree_t, typename Config::geometry_t, typename Config::equation_t, Config::DIM> solver(
        2000, 1.0, 0.4);
    const std::array<double, 2> start_pos = { 0.2, 0.2 };
    auto ic = [&](auto const& coords) -> amr::containers::static_vector<double, 1> {
        double r2 = 0.0;
        for (int d = 0; d < Config::DIM; ++d) r2 += std::pow(coords[d] - start_pos[d], 2);
        return { std::exp(-r2 / 0.005) };
    };
    solver.initialize(ic);
    double t = 0.0, dt = 0.0, t_target = 0.5;
    while (t < t_target) {
        dt = solver.advance();
        if (t + dt > t_target) dt = t_target - t;
        solver.get_tree().halo_exchange_update();
        t += dt;
    }
    std::array<double, Config::DIM> expected_pos;
    for (int d = 0; d < Config::DIM; ++d)
        expected_pos[d] = start_pos[d] + Config::equation_t::Velocity[d] * t_target;
    std::array<double, 2> actual_pos{};
    find_peak<Config>(solver.get_tree(), actual_pos);
    auto cell_size = Config::geometry_t::cell_sizes(solver.get_tree().get_node_index_at(0));
    for (int d = 0; d < Config::DIM; ++d) EXPECT_NEAR(actual_pos[d], expected_pos[d], cell_size[d]);
}

template <typename Config>
void PulseCenterMovementAMR()
{
    amr_solver<typename Config::tree_t, typename Config::geometry_t, typename Config::equation_t, Config::DIM> solver(
        2000, 1.0, 0.4);
    const std::array<double, 2> start_pos = { 0.2, 0.2 };
    auto ic = [&](auto const& coords) -> amr::containers::static_vector<double, 1> {
        double r2 = 0.0;
        for (int d = 0; d < Config::DIM; ++d) r2 += std::pow(coords[d] - start_pos[d], 2);
        return { std::exp(-r2 / 0.005) };
    };
    auto amrCriterion = [&](const typename Config::patch_index_t& idx) {
        auto   patch   = solver.get_tree().template get_patch<amr::cell::Scalar>(idx);
        auto&  data    = patch.data();
        double max_val = 0;
        for (auto v : data) max_val = std::max(max_val, v);
        if (max_val > 0.1 && idx.level() < 5) return Config::tree_t::refine_status_t::Refine;
        if (max_val < 0.05 && idx.level() > 1) return Config::tree_t::refine_status_t::Coarsen;
        return Config::tree_t::refine_status_t::Stable;
    };
    solver.initialize(ic);
    solver.get_tree().halo_exchange_update();
    double t = 0.0, t_target = 0.5;
    while (t < t_target) {
        const double dt = solver.advance();
        solver.get_tree().halo_exchange_update();
        solver.get_tree().reconstruct_tree(amrCriterion);
        solver.get_tree().halo_exchange_update();
        t += dt;
    }
    std::array<double, Config::DIM> expected_pos;
    for (int d = 0; d < Config::DIM; ++d)
        expected_pos[d] = start_pos[d] + Config::equation_t::Velocity[d] * t_target;
    std::array<double, 2> actual_pos{};
    find_peak<Config>(solver.get_tree(), actual_pos);
    auto cell_size = Config::geometry_t::cell_sizes(solver.get_tree().get_node_index_at(0));
    for (int d = 0; d < Config::DIM; ++d) EXPECT_NEAR(actual_pos[d], expected_pos[d], cell_size[d]);
}

// ---------------------------------------------------------------- config 2
static std::uint64_t mix64(std::uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static double unit_hash(std::uint64_t a, std::uint64_t b, std::uint64_t c)
{
    return static_cast<double>(mix64(a ^ mix64(b ^ mix64(c))) >> 11) * 0x1.0p-53;
}

int bench_loop(int argc, char** argv)
{
    // argv: steps remesh noise seed b0x b0y b0s b0a b1x b1y b1s b1a
    using shape_t        = amr::containers::static_shape<16u, 16u>;
    using layout_t       = amr::containers::static_layout<shape_t>;
    using patch_index_t  = amr::ndt::morton::morton_id<7u, 2u>;
    using patch_layout_t = amr::ndt::patches::patch_layout<layout_t, 1>;
    using interp_t       = amr::ndt::intergrid_operator::linear_interpolator<patch_layout_t>;
    using tree_t         = amr::ndt::tree::ndtree<amr::cell::AdvectionCell, patch_index_t, patch_layout_t, interp_t>;
    static constexpr std::array<double, 2> lengths = { 1.0, 1.0 };
    using physics_t = amr::ndt::solver::physics_system<patch_index_t, patch_layout_t, lengths>;
    const long   steps = std::atol(argv[2]), interval = std::atol(argv[3]);
    const double noise = std::atof(argv[4]);
    const auto   seed  = static_cast<std::uint64_t>(std::atoll(argv[5]));
    double       b[8];
    for (int i = 0; i < 8; ++i) b[i] = std::atof(argv[6 + i]);
    (void)argc;

    amr_solver<tree_t, physics_t, AdvectionPhysics<2>, 2> solver(20000, 1.0, 0.4);
    auto refine_all = [](patch_index_t const&) { return tree_t::refine_status_t::Refine; };
    for (int i = 0; i < 2; ++i) {
        solver.get_tree().reconstruct_tree(refine_all);
        solver.get_tree().halo_exchange_update();
    }
    solver.initialize([&](auto const& x) -> amr::containers::static_vector<double, 1> {
        double v = 0.0;
        for (int k = 0; k < 2; ++k) {
            double r2 = 0.0;
            for (int d = 0; d < 2; ++d) {
                const double diff = x[d] - b[4 * k + d];
                r2 += diff * diff;
            }
            const double s = b[4 * k + 2], a = b[4 * k + 3];
            v += a * std::exp(-r2 / (2.0 * s * s));
        }
        return { v };
    });
    auto& tree = solver.get_tree();
    for (std::size_t p = 0; p < tree.size(); ++p) {
        const auto    id   = tree.get_node_index_at(p).id();
        auto&         u    = tree.template get_patch<amr::cell::Scalar>(p);
        std::uint64_t cell = 0;
        for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li) {
            if (amr::ndt::utils::patches::is_halo_cell<patch_layout_t>(li)) continue;
            u[li] += noise * (2.0 * unit_hash(seed, id, cell) - 1.0);
            ++cell;
        }
    }
    tree.sync_current_to_device();
    tree.halo_exchange_update();
    const amr::gb300::gradient_criterion crit{ 0.05, 0.01, 1, 5 };
    double      t = 0.0;
    long        done = 0;
    std::size_t cells = 0;
    while (done < steps) {
        const long  k      = std::min(interval, steps - done);
        const auto  before = tree.size();
        solver.advance_batch_async(static_cast<std::size_t>(k));
        tree.reconstruct_tree(crit);
        tree.halo_exchange_update();
        std::size_t executed = 0;
        t += solver.finish_advance_batch(&executed);
        cells += executed * before * 256;
        done += static_cast<long>(executed);
    }
    std::printf("sum_dt %.17g steps %ld cells %zu leaves %zu\n", t, done, cells, tree.size());
    for (std::size_t p = 0; p < tree.size(); ++p) std::printf("id %llu\n", (unsigned long long)tree.get_node_index_at(p).id());
    for (std::size_t p = 0; p < tree.size(); ++p) {
        auto const& u = tree.template get_patch<amr::cell::Scalar>(p);
        for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li)
            if (!amr::ndt::utils::patches::is_halo_cell<patch_layout_t>(li)) std::printf("u %.17g\n", u[li]);
    }
    return 0;
}

// The Euler benchmark written against the reference's API: amr_solver with
// EulerPhysics2D, initialize() with the acoustic pulse, a host criterion on
// the Rho patches through reconstruct_tree, the advance/re-mesh/halo loop.
// argv: steps remesh init_levels min_level max_level.  Prints the initial and
// final state (interior and face-ghost cells, field by field), the ids, the
// simulated time and the executed steps.
int euler_loop(int argc, char** argv)
{
    using shape_t        = amr::containers::static_shape<8u, 8u>;
    using layout_t       = amr::containers::static_layout<shape_t>;
    using patch_index_t  = amr::ndt::morton::morton_id<7u, 2u>;
    using patch_layout_t = amr::ndt::patches::patch_layout<layout_t, 1>;
    using interp_t       = amr::ndt::intergrid_operator::linear_interpolator<patch_layout_t>;
    using tree_t         = amr::ndt::tree::ndtree<amr::cell::EulerCell2D, patch_index_t, patch_layout_t, interp_t>;
    static constexpr std::array<double, 2> lengths = { 1000.0, 1000.0 };
    using physics_t = amr::ndt::solver::physics_system<patch_index_t, patch_layout_t, lengths>;
    (void)argc;
    const long steps = std::atol(argv[2]), interval = std::atol(argv[3]);
    const int  init = std::atoi(argv[4]), min_level = std::atoi(argv[5]), max_level = std::atoi(argv[6]);

    amr_solver<tree_t, physics_t, EulerPhysics2D, 2> solver(20000, 1.4, 0.3);
    auto& tree       = solver.get_tree();
    auto  refine_all = [](patch_index_t const&) { return tree_t::refine_status_t::Refine; };
    for (int i = 0; i < init; ++i) {
        tree.reconstruct_tree(refine_all);
        tree.halo_exchange_update();
    }
    // acoustic pulse: rho = 0.5 + 0.2 A e, p = 1 + A e, e = exp(-r^2 / w^2)
    const double amp = 10.0, width_sq = 0.01 * lengths[0] * lengths[1];
    solver.initialize([&](auto const& x) -> amr::containers::static_vector<double, 4> {
        const double dx = x[0] - 0.5 * lengths[0], dy = x[1] - 0.5 * lengths[1];
        const double e  = amp * std::exp(-(dx * dx + dy * dy) / width_sq);
        return { 0.5 + (e * 0.2), 0.0, 0.0, 1.0 + e };
    });
    tree.sync_current_to_device();
    tree.halo_exchange_update();
    auto print_state = [&](const char* tag) {
        const auto faces = [](std::size_t li) {
            int outside = 0;
            for (int k = 0; k < 2; ++k, li /= 10) outside += (li % 10 == 0 || li % 10 == 9) ? 1 : 0;
            return outside <= 1;
        };
        for (std::size_t f = 0; f < 4; ++f)
            for (std::size_t p = 0; p < tree.size(); ++p) {
                auto const& u = tree.get_field_patch(f, p);
                for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li)
                    if (faces(li)) std::printf("%s %.17g\n", tag, u[li]);
            }
    };
    print_state("s0");
    // the benchmark's criterion, evaluated on the host over the Rho patch
    struct rho_criterion
    {
        tree_t& t;
        double  rthr, cthr;
        int     minl, maxl;
        auto operator()(patch_index_t const& idx) const -> tree_t::refine_status_t
        {
            auto const& rho = t.template get_patch<amr::cell::Rho>(idx);
            double      m   = 0.0;
            for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li) m = std::max(rho[li], m);
            if (idx.level() < maxl && m > rthr) return tree_t::refine_status_t::Refine;
            if (idx.level() > minl && m < cthr) return tree_t::refine_status_t::Coarsen;
            return tree_t::refine_status_t::Stable;
        }
    };
    const rho_criterion crit{ tree, 0.53, 0.49, min_level, max_level };
    double t = 0.0;
    long   done = 0;
    while (done < steps) {
        solver.advance_batch_async(static_cast<std::size_t>(std::min(interval, steps - done)));
        tree.reconstruct_tree(crit);
        tree.halo_exchange_update();
        std::size_t executed = 0;
        t += solver.finish_advance_batch(&executed);
        done += static_cast<long>(executed);
        if (executed == 0) break;
    }
    std::printf("time %.17g steps %ld leaves %zu\n", t, done, tree.size());
    for (std::size_t p = 0; p < tree.size(); ++p) std::printf("id %llu\n", (unsigned long long)tree.get_node_index_at(p).id());
    print_state("s1");
    return 0;
}

// The adjoint through the C++ header: dot-product identity
// <lambda_T, A u_0> = <A^T lambda_T, u_0> over interior cells on a 2:1 mesh.
static int adjoint_check()
{
    amr_tree_desc d{};
    d.geom.rank = 2;
    d.geom.n = 16;
    d.geom.halo = 1;
    d.geom.depth = 6;
    d.geom.lengths[0] = d.geom.lengths[1] = d.geom.lengths[2] = 1.0;
    d.capacity = 4096;
    d.dtype    = AMR_F64;
    amr_tree* t = nullptr;
    amr::gb300::check(amr_tree_create(&d, &t));
    amr::gb300::check(amr_tree_refine_uniform(t, 2));
    std::size_t P = 0, flat = 0;
    amr::gb300::check(amr_tree_size(t, &P));
    std::vector<std::int8_t> f(P, 0);
    f[0] = f[5] = f[9] = 1;
    amr::gb300::check(amr_tree_set_flags(t, f.data(), P));
    int changed = 0;
    amr::gb300::check(amr_tree_remesh(t, &changed));
    amr::gb300::check(amr_tree_size(t, &P));
    amr::gb300::check(amr_tree_patch_cells(t, &flat));
    std::vector<double> u0(P * flat), lt(P * flat), l0(P * flat), ut(P * flat);
    for (std::size_t i = 0; i < u0.size(); ++i) {
        u0[i] = unit_hash(1, i, 0) - 0.5;
        lt[i] = unit_hash(2, i, 0) - 0.5;
    }
    amr::gb300::check(amr_tree_upload_state(t, u0.data(), P));
    double lhs = 0.0, rhs = 0.0;
    {
        amr::gb300::adjoint adj(t, 17, { 1.0, -0.5, 0.0 }, 0.4, 5);
        adj.forward();
        amr::gb300::check(amr_tree_download_state(t, ut.data(), P));
        adj.backward_host(lt.data(), l0.data());
        if (adj.checkpoints() != 5) ++g_failures;
    }
    for (std::size_t p = 0; p < P; ++p)
        for (int r = 1; r <= 16; ++r)
            for (int c = 1; c <= 16; ++c) {
                const std::size_t i = p * flat + r * 18 + c;
                lhs += lt[i] * ut[i];
                rhs += l0[i] * u0[i];
            }
    EXPECT_NEAR(lhs, rhs, 1e-12 * std::abs(lhs));
    amr_tree_destroy(t);
    std::cout << (g_failures ? "FAILED" : "PASSED") << " " << g_failures << "\n";
    return g_failures ? 1 : 0;
}

int main(int argc, char** argv)
{
    const std::string mode = argc > 1 ? argv[1] : "tests";
    if (mode == "bench") return bench_loop(argc, argv);
    if (mode == "adjoint") return adjoint_check();
    if (mode == "euler") return euler_loop(argc, argv);
    PulseCenterMovement<AdvectionTestConfig<2, 10>>();
    PulseCenterMovement<AdvectionTestConfig<2, 50>>();
    PulseCenterMovementAMR<AdvectionTestConfig<2, 10>>();
    PulseCenterMovementAMR<AdvectionTestConfig<2, 50>>();
    std::cout << (g_failures ? "FAILED" : "PASSED") << " " << g_failures << "\n";
    return g_failures ? 1 : 0;
}
