// Test infrastructure only: a driver that runs the UNMODIFIED gpu-amr reference
// (header-only C++23, compiled from its own sources by oracle/Makefile into
// oracle/_ref/) and dumps its tree, flags and cell states as binary records.
// The dumps become the golden fixtures under tests/golden/ that pin both the
// C restatement in oracle/ and the CUDA path.  Nothing shipped links this file.
//
// Reference entry points exercised (paths within the reference project):
//   amr_solver::initialize / advance_batch_async / finish_advance_batch
//       include/solver/amr_solver.hpp:105-262
//   ndtree::reconstruct_tree, halo_exchange_update, get_neighbor_at
//       include/ndtree/ndtree.hpp:1249-1271, 1862-1877, 682-689
//   physics_system::cell_coord / cell_sizes  include/solver/physics_system.hpp:75-138
//
// Harness plug-ins (same static interface as the reference's own plug-ins):
//   RuntimeAdvection  - AdvectionPhysics (include/solver/AdvectionPhysics.hpp:17-91)
//                       with the velocity read from a runtime array; the flux
//                       expression is the reference's, term for term.
//   gradient criterion - max|grad u|*h with the any/all patch rule of
//                       include/dg_helpers/globals/amr_indicators.hpp:186-225.
//   max criterion      - the max-value rule of tests/advection_equation_amr.t.cpp:155-170.
//   random criterion   - hash-driven flags for tree-operation coverage.
//   mode=euler          - the reference's amr_solver with EulerPhysics<DIM>
//                       on the acoustic pulse of its Euler benchmark
//                       (benchmark/bench_fvm_solver_integration.b.cpp:
//                       95-178: domain 1000^DIM, max-Rho criterion over the
//                       padded patch, re-mesh every `remesh` steps).
//   mode=ssprk order=2|3 - the reference's SSPRK2 / SSPRK3 classes
//                       (include/dg_helpers/time_integration/time.hpp) driving
//                       the FV advection residual -sum_d (F_R - F_L)/dx_d
//                       (RuntimeAdvection's Rusanov flux) patch by patch, with
//                       a halo exchange before every stage as the DG solver
//                       does (include/dg_helpers/solver.hpp:162-244); CFL step
//                       as compute_time_step_cpu; gradient re-mesh as in run.
//   vtk=<name>          - after the mode, the reference's VTK writer
//                       (include/ndtree/vtk_print.hpp) prints the tree to
//                       vtk_output/<name>.vtk.
#include "containers/static_layout.hpp"
#include "containers/static_shape.hpp"
#include "containers/static_vector.hpp"
#include "morton/morton_id.hpp"
#include "ndtree/intergrid_operator.hpp"
#include "ndtree/ndtree.hpp"
#include "ndtree/patch_layout.hpp"
#include "ndtree/vtk_print.hpp"
#include "containers/container_operations.hpp"
#include "dg_helpers/time_integration/time.hpp"
#include "solver/EulerPhysics.hpp"
#include "solver/amr_solver.hpp"
#include "solver/cell_types.hpp"
#include "solver/physics_system.hpp"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace harness
{

// ---------------------------------------------------------------- hashing
// SplitMix64 finaliser; the same function is restated in oracle/amr_oracle.c
// and in the product's host initialiser so all three draw identical noise.
static inline std::uint64_t mix64(std::uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static inline double unit_hash(std::uint64_t a, std::uint64_t b, std::uint64_t c)
{
    const std::uint64_t h = mix64(a ^ mix64(b ^ mix64(c)));
    return static_cast<double>(h >> 11) * 0x1.0p-53;
}

// ---------------------------------------------------------------- params
struct params
{
    std::map<std::string, std::string> kv;

    auto has(const char* k) const -> bool { return kv.count(k) != 0; }
    auto str(const char* k, const char* d) const -> std::string
    {
        auto it = kv.find(k);
        return it == kv.end() ? std::string(d) : it->second;
    }
    auto num(const char* k, double d) const -> double
    {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::strtod(it->second.c_str(), nullptr);
    }
    auto integer(const char* k, long d) const -> long
    {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::strtol(it->second.c_str(), nullptr, 10);
    }
    auto list(const char* k) const -> std::vector<double>
    {
        std::vector<double> out;
        auto                s = str(k, "");
        const char*         p = s.c_str();
        while (*p)
        {
            char* end = nullptr;
            out.push_back(std::strtod(p, &end));
            if (end == p) break;
            p = end;
            while (*p == ',' || *p == ';') ++p;
        }
        return out;
    }
};

// ---------------------------------------------------------------- writer
struct writer
{
    std::FILE* f = nullptr;
    explicit writer(const std::string& path)
    {
        f = std::fopen(path.c_str(), "wb");
        if (!f)
        {
            std::perror(path.c_str());
            std::exit(2);
        }
    }
    ~writer() { std::fclose(f); }
    template <typename T>
    void put(T const& v) { std::fwrite(&v, sizeof(T), 1, f); }
    void bytes(const void* p, std::size_t n) { std::fwrite(p, 1, n, f); }
    void header(std::uint32_t tag, std::uint32_t step, std::uint64_t payload)
    {
        put(tag);
        put(step);
        put(payload);
    }
};

enum : std::uint32_t
{
    TAG_TREE  = 1,
    TAG_FLAGS = 2,
    TAG_STATE = 3,
    TAG_DT    = 4,
};

// Runtime velocity for the harness equation.
inline double g_velocity[3] = { 1.0, 0.5, 0.0 };

template <int DIM>
struct RuntimeAdvection
{
    static constexpr int NVAR = 1;
    using FieldTags           = std::tuple<amr::cell::Scalar>;

    static void primitiveToConservative(
        const amr::containers::static_vector<double, NVAR>& prim,
        amr::containers::static_vector<double, NVAR>&       cons,
        double
    )
    {
        cons[0] = prim[0];
    }

    static void rusanovFlux(
        const amr::containers::static_vector<double, NVAR>& UL,
        const amr::containers::static_vector<double, NVAR>& UR,
        amr::containers::static_vector<double, NVAR>&       flux,
        int                                                 direction,
        double
    )
    {
        double fluxL = UL[0] * g_velocity[direction];
        double fluxR = UR[0] * g_velocity[direction];
        double smax  = std::abs(g_velocity[direction]);
        flux[0]      = 0.5 * (fluxL + fluxR) - 0.5 * smax * (UR[0] - UL[0]);
    }

    template <typename PatchTuple>
    static double getMaxSpeed(const PatchTuple&, std::size_t, int direction, double)
    {
        return std::abs(g_velocity[direction]);
    }
};

// TAG_TREE record of a tree: per leaf its Morton id and, per direction, the
// neighbour variant (kind, contact quadrant, ids).
template <int DIM, typename Tree>
void dump_tree_records(Tree& t, writer& W, std::uint32_t step)
{
    using dir_t                  = typename Tree::patch_direction_t;
    const std::uint64_t n        = t.size();
    const std::uint64_t per_dir  = 4 + 4 + 4 * 8;
    W.header(TAG_TREE, step, 8 + n * (8 + 2 * DIM * per_dir));
    W.put(n);
    for (std::size_t i = 0; i != n; ++i)
    {
        W.put(static_cast<std::uint64_t>(t.get_node_index_at(i).id()));
        for (auto d = dir_t::first(); d != dir_t::sentinel(); d.advance())
        {
            const auto    nb     = t.get_neighbor_at(i, d);
            std::uint8_t  kind   = 0;
            std::uint8_t  q[3]   = { 0, 0, 0 };
            std::uint64_t ids[4] = { 0, 0, 0, 0 };
            using nv_t           = std::remove_cvref_t<decltype(nb)>;
            std::visit(
                [&](auto const& v)
                {
                    using V = std::remove_cvref_t<decltype(v)>;
                    if constexpr (std::is_same_v<V, typename nv_t::none>)
                    {
                        kind = 0;
                    }
                    else if constexpr (std::is_same_v<V, typename nv_t::same>)
                    {
                        kind   = 1;
                        ids[0] = v.id.id();
                    }
                    else if constexpr (std::is_same_v<V, typename nv_t::finer>)
                    {
                        kind = 2;
                        for (std::size_t k = 0; k != v.ids.size(); ++k) ids[k] = v.ids[k].id();
                    }
                    else
                    {
                        kind   = 3;
                        ids[0] = v.id.id();
                        for (std::size_t k = 0; k != v.contact_quadrant.size(); ++k)
                            q[k] = static_cast<std::uint8_t>(v.contact_quadrant[k]);
                    }
                },
                nb.data
            );
            W.put(kind);
            W.bytes(q, 3);
            W.put(std::uint32_t{ 0 });
            W.bytes(ids, sizeof(ids));
        }
    }
}

template <int DIM, std::size_t N, std::size_t H, unsigned Depth>
struct harness
{
    using shape_t = std::conditional_t<
        DIM == 2,
        amr::containers::static_shape<N, N>,
        amr::containers::static_shape<N, N, N>>;
    using layout_t       = amr::containers::static_layout<shape_t>;
    using patch_index_t  = amr::ndt::morton::morton_id<Depth, unsigned(DIM)>;
    using patch_layout_t = amr::ndt::patches::patch_layout<layout_t, H>;
    using interp_t = amr::ndt::intergrid_operator::linear_interpolator<patch_layout_t>;
    using tree_t   = amr::ndt::tree::
        ndtree<amr::cell::AdvectionCell, patch_index_t, patch_layout_t, interp_t>;
    static constexpr std::array<double, DIM> lengths = [] {
        std::array<double, DIM> l{};
        for (auto& e : l) e = 1.0;
        return l;
    }();
    using geometry_t = amr::ndt::solver::physics_system<patch_index_t, patch_layout_t, lengths>;
    using solver_t   = amr_solver<tree_t, geometry_t, RuntimeAdvection<DIM>, DIM>;
    using padded_t   = typename patch_layout_t::padded_layout_t;
    using status_t   = typename tree_t::refine_status_t;
    using dir_t      = typename tree_t::patch_direction_t;

    static constexpr std::size_t flat    = patch_layout_t::flat_size();
    static constexpr std::size_t padded1 = N + 2 * H;

    params const& P;
    writer&       W;
    solver_t      solver;
    std::vector<std::int8_t> last_flags;

    harness(params const& p, writer& w)
        : P(p), W(w), solver(static_cast<std::size_t>(p.integer("capacity", 20000)), 1.0, p.num("cfl", 0.4))
    {
    }

    auto tree() -> tree_t& { return solver.get_tree(); }

    // ---- dumps
    void dump_tree(std::uint32_t step) { dump_tree_records<DIM>(tree(), W, step); }

    void dump_flags(std::uint32_t step)
    {
        const std::uint64_t n = last_flags.size();
        W.header(TAG_FLAGS, step, 8 + n);
        W.put(n);
        W.bytes(last_flags.data(), n);
    }

    void dump_state(std::uint32_t step)
    {
        auto&               t = tree();
        const std::uint64_t n = t.size();
        W.header(TAG_STATE, step, 16 + n * flat * 8);
        W.put(n);
        W.put(static_cast<std::uint64_t>(flat));
        for (std::size_t i = 0; i != n; ++i)
        {
            auto const& p = t.template get_patch<amr::cell::Scalar>(i);
            for (std::size_t c = 0; c != flat; ++c)
            {
                double v = p[static_cast<typename padded_t::index_t>(c)];
                W.put(v);
            }
        }
    }

    // ---- initial data
    void init_state()
    {
        auto                bumps = P.list("bumps");
        const int           per   = DIM + 2;
        const double        noise = P.num("noise", 0.0);
        const std::uint64_t seed  = static_cast<std::uint64_t>(P.integer("noise_seed", 0));
        auto ic = [&](auto const& x) -> amr::containers::static_vector<double, 1>
        {
            double v = 0.0;
            for (std::size_t b = 0; b + per <= bumps.size(); b += per)
            {
                double r2 = 0.0;
                for (int d = 0; d < DIM; ++d)
                {
                    const double diff = x[d] - bumps[b + d];
                    r2 += diff * diff;
                }
                const double s   = bumps[b + DIM];
                const double amp = bumps[b + DIM + 1];
                v += amp * std::exp(-r2 / (2.0 * s * s));
            }
            return { v };
        };
        solver.initialize(ic);
        if (noise != 0.0)
        {
            auto& t = tree();
            for (std::size_t i = 0; i != t.size(); ++i)
            {
                auto&             p  = t.template get_patch<amr::cell::Scalar>(i);
                const std::uint64_t id = t.get_node_index_at(i).id();
                std::uint64_t     cell = 0;
                amr::containers::manipulators::shaped_for<
                    typename patch_layout_t::interior_iteration_control_t>(
                    [&](auto const& idxs)
                    {
                        const auto li = padded_t::linear_index(idxs);
                        p[li] += noise * (2.0 * unit_hash(seed, id, cell) - 1.0);
                        ++cell;
                    }
                );
            }
        }
    }

    void random_state(std::uint64_t seed)
    {
        auto& t = tree();
        for (std::size_t i = 0; i != t.size(); ++i)
        {
            auto&               p  = t.template get_patch<amr::cell::Scalar>(i);
            const std::uint64_t id = t.get_node_index_at(i).id();
            for (std::size_t c = 0; c != flat; ++c)
                p[static_cast<typename padded_t::index_t>(c)] = unit_hash(seed, id, c) - 0.5;
        }
    }

    // ---- criteria
    static auto level_of(patch_index_t const& idx) -> int { return static_cast<int>(idx.level()); }

    auto gradient_status(patch_index_t const& idx) -> status_t
    {
        const double rthr  = P.num("rthr", 0.05);
        const double cthr  = P.num("cthr", 0.01);
        const int    minl  = static_cast<int>(P.integer("min_level", 1));
        const int    maxl  = static_cast<int>(P.integer("max_level", 5));
        auto const&  p     = tree().template get_patch<amr::cell::Scalar>(idx);
        const std::size_t sy = padded1;
        const std::size_t sz = padded1 * padded1;
        bool any_refine = false;
        bool all_coarsen = true;
        amr::containers::manipulators::shaped_for<
            typename patch_layout_t::interior_iteration_control_t>(
            [&](auto const& idxs)
            {
                const std::size_t li = padded_t::linear_index(idxs);
                double s = 0.0;
                for (int d = 0; d < DIM; ++d)
                {
                    const std::size_t st = d == 0 ? 1 : (d == 1 ? sy : sz);
                    const double g = 0.5 * (p[static_cast<typename padded_t::index_t>(li + st)] -
                                            p[static_cast<typename padded_t::index_t>(li - st)]);
                    s += g * g;
                }
                const double v = std::sqrt(s);
                if (v > rthr) any_refine = true;
                if (!(v < cthr)) all_coarsen = false;
            }
        );
        const int level = level_of(idx);
        if (level < maxl && any_refine) return status_t::Refine;
        if (level > minl && all_coarsen) return status_t::Coarsen;
        return status_t::Stable;
    }

    auto max_status(patch_index_t const& idx) -> status_t
    {
        const double rthr = P.num("rthr", 0.1);
        const double cthr = P.num("cthr", 0.05);
        const int    minl = static_cast<int>(P.integer("min_level", 1));
        const int    maxl = static_cast<int>(P.integer("max_level", 5));
        auto const&  p    = tree().template get_patch<amr::cell::Scalar>(idx);
        double       m    = 0.0;
        for (std::size_t c = 0; c != flat; ++c)
            m = std::max(m, p[static_cast<typename padded_t::index_t>(c)]);
        const int level = level_of(idx);
        if (m > rthr && level < maxl) return status_t::Refine;
        if (m < cthr && level > minl) return status_t::Coarsen;
        return status_t::Stable;
    }

    auto random_status(patch_index_t const& idx, std::uint64_t seed, std::uint64_t pass)
        -> status_t
    {
        const double pr   = P.num("p_refine", 0.2);
        const double pc   = P.num("p_coarsen", 0.5);
        const int    minl = static_cast<int>(P.integer("min_level", 1));
        const int    maxl = static_cast<int>(P.integer("max_level", 5));
        const int    level = level_of(idx);
        const double u1    = unit_hash(seed, pass, idx.id());
        if (u1 < pr && level < maxl) return status_t::Refine;
        if (level > 0)
        {
            const auto   parent = patch_index_t::parent_of(idx);
            const double u2     = unit_hash(seed ^ 0x5bd1e995ull, pass, parent.id());
            if (u2 < pc && level > minl) return status_t::Coarsen;
        }
        return status_t::Stable;
    }

    template <typename Fn>
    void remesh(Fn&& fn)
    {
        last_flags.clear();
        auto recording = [&](patch_index_t const& idx) -> status_t
        {
            const auto s = fn(idx);
            last_flags.push_back(static_cast<std::int8_t>(s));
            return s;
        };
        tree().reconstruct_tree(recording);
        tree().halo_exchange_update();
    }

    void uniform_refine(int levels)
    {
        auto refine_all = [](patch_index_t const&) { return status_t::Refine; };
        for (int i = 0; i < levels; ++i)
        {
            tree().reconstruct_tree(refine_all);
            tree().halo_exchange_update();
        }
    }

    // ---- modes
    int run()
    {
        auto vel = P.list("vel");
        for (std::size_t d = 0; d < vel.size() && d < 3; ++d) g_velocity[d] = vel[d];
        uniform_refine(static_cast<int>(P.integer("init_levels", 2)));
        init_state();
        tree().halo_exchange_update();
        dump_tree(0);
        dump_state(0);

        const long        steps       = P.integer("steps", 100);
        const long        interval    = P.integer("remesh", 0);
        const long        state_every = P.integer("state_every", 0);
        const std::string crit        = P.str("crit", "none");
        long              done        = 0;
        long              batch       = 0;
        double            sum_dt      = 0.0;
        std::uint64_t     cell_updates = 0;
        const auto        t0 = std::chrono::steady_clock::now();
        while (done < steps)
        {
            const long k = interval > 0 ? std::min(interval, steps - done) : steps - done;
            const auto leaves = tree().size();
            solver.advance_batch_async(static_cast<std::size_t>(k));
            std::size_t executed = 0;
            sum_dt += solver.finish_advance_batch(&executed);
            cell_updates += executed * leaves * layout_t::flat_size();
            done += static_cast<long>(executed);
            ++batch;
            if (interval > 0 && crit != "none")
            {
                if (state_every > 0 && batch % state_every == 0)
                    dump_state(static_cast<std::uint32_t>(done));
                if (crit == "grad")
                    remesh([&](patch_index_t const& i) { return gradient_status(i); });
                else
                    remesh([&](patch_index_t const& i) { return max_status(i); });
                dump_flags(static_cast<std::uint32_t>(done));
                dump_tree(static_cast<std::uint32_t>(done));
            }
            if (executed == 0) break;
        }
        const auto t1 = std::chrono::steady_clock::now();
        const double secs = std::chrono::duration<double>(t1 - t0).count();
        dump_state(static_cast<std::uint32_t>(done));
        W.header(TAG_DT, static_cast<std::uint32_t>(done), 16);
        W.put(sum_dt);
        W.put(static_cast<std::uint64_t>(done));
        std::printf(
            "{\"steps\": %ld, \"sum_dt\": %.17g, \"leaves\": %zu, \"cell_updates\": %llu, "
            "\"seconds\": %.6f, \"cell_updates_per_s\": %.6e}\n",
            done, sum_dt, tree().size(), static_cast<unsigned long long>(cell_updates), secs,
            static_cast<double>(cell_updates) / secs
        );
        return 0;
    }

    // ---- SSPRK (mode=ssprk)
    using container_t = amr::containers::static_tensor<double, padded_t>;

    // compute_time_step_cpu (amr_solver.hpp:355-413) for the advection speeds
    auto cfl_dt(double cfl) -> double
    {
        double dt = std::numeric_limits<double>::max();
        auto&  t  = tree();
        for (std::size_t i = 0; i != t.size(); ++i)
        {
            const auto cs = geometry_t::cell_sizes(t.get_node_index_at(i));
            for (int d = 0; d < DIM; ++d)
            {
                const double speed = std::abs(g_velocity[d]);
                if (speed > 1e-12) dt = std::min(dt, cs[d] / speed);
            }
        }
        return cfl * dt;
    }

    template <typename Integrator>
    void ssprk_step(double dt)
    {
        auto&             t = tree();
        const std::size_t n = t.size();
        std::vector<Integrator> integ(n);
        t.halo_exchange_update();
        for (std::size_t i = 0; i != n; ++i) integ[i].begin_step(t.template get_patch<amr::cell::Scalar>(i).data());
        for (int s = 0; s < Integrator::num_stages(); ++s)
        {
            t.halo_exchange_update();
            for (std::size_t i = 0; i != n; ++i)
            {
                auto&      patch = t.template get_patch<amr::cell::Scalar>(i);
                const auto cs    = geometry_t::cell_sizes(t.get_node_index_at(i));
                auto residual = [&](container_t& update, const container_t& cur, double)
                {
                    amr::containers::manipulators::shaped_for<
                        typename patch_layout_t::interior_iteration_control_t>(
                        [&](auto const& idxs)
                        {
                            const std::size_t li = padded_t::linear_index(idxs);
                            double            R  = 0.0;
                            for (int d = 0; d < DIM; ++d)
                            {
                                const std::size_t st = d == 0 ? 1 : (d == 1 ? padded1 : padded1 * padded1);
                                using sv             = amr::containers::static_vector<double, 1>;
                                sv UL, UC, UR, fL, fR;
                                UL[0] = cur[static_cast<typename padded_t::index_t>(li - st)];
                                UC[0] = cur[static_cast<typename padded_t::index_t>(li)];
                                UR[0] = cur[static_cast<typename padded_t::index_t>(li + st)];
                                RuntimeAdvection<DIM>::rusanovFlux(UL, UC, fL, d, 0.0);
                                RuntimeAdvection<DIM>::rusanovFlux(UC, UR, fR, d, 0.0);
                                R -= (fR[0] - fL[0]) / cs[d];
                            }
                            update[static_cast<typename padded_t::index_t>(li)] = R;
                        }
                    );
                };
                integ[i].compute_stage(s, residual, patch.data(), 0.0, dt);
                patch.data() = integ[i].stage_result(s, patch.data());
            }
        }
        for (std::size_t i = 0; i != n; ++i) integ[i].finish_step(t.template get_patch<amr::cell::Scalar>(i).data());
    }

    int ssprk_mode()
    {
        auto vel = P.list("vel");
        for (std::size_t d = 0; d < vel.size() && d < 3; ++d) g_velocity[d] = vel[d];
        uniform_refine(static_cast<int>(P.integer("init_levels", 2)));
        init_state();
        tree().halo_exchange_update();
        dump_tree(0);
        dump_state(0);
        const int    order    = static_cast<int>(P.integer("order", 2));
        const long   steps    = P.integer("steps", 40);
        const long   interval = P.integer("remesh", 10);
        const double cfl      = P.num("cfl", 0.4);
        double       sum_dt   = 0.0;
        double       batch    = 0.0; // steps since the last re-mesh, added like finish_advance_batch
        for (long s = 1; s <= steps; ++s)
        {
            const double dt = cfl_dt(cfl);
            if (order == 3)
                ssprk_step<amr::time_integration::SSPRK3<container_t>>(dt);
            else
                ssprk_step<amr::time_integration::SSPRK2<container_t>>(dt);
            batch += dt;
            if ((interval > 0 && s % interval == 0) || s == steps)
            {
                sum_dt += batch;
                batch = 0.0;
            }
            if (interval > 0 && s % interval == 0)
            {
                remesh([&](patch_index_t const& i) { return gradient_status(i); });
                dump_flags(static_cast<std::uint32_t>(s));
                dump_tree(static_cast<std::uint32_t>(s));
            }
        }
        tree().halo_exchange_update();
        dump_state(static_cast<std::uint32_t>(steps));
        W.header(TAG_DT, static_cast<std::uint32_t>(steps), 16);
        W.put(sum_dt);
        W.put(static_cast<std::uint64_t>(steps));
        std::printf("{\"steps\": %ld, \"sum_dt\": %.17g, \"leaves\": %zu}\n", steps, sum_dt, tree().size());
        return 0;
    }

    int tree_mode()
    {
        const std::uint64_t seed   = static_cast<std::uint64_t>(P.integer("seed", 1));
        const long          passes = P.integer("passes", 4);
        uniform_refine(static_cast<int>(P.integer("init_levels", 2)));
        random_state(seed * 7919u + 17u);
        tree().halo_exchange_update();
        dump_tree(0);
        dump_state(0);
        for (long pass = 1; pass <= passes; ++pass)
        {
            remesh([&](patch_index_t const& i)
                   { return random_status(i, seed, static_cast<std::uint64_t>(pass)); });
            dump_flags(static_cast<std::uint32_t>(pass));
            dump_tree(static_cast<std::uint32_t>(pass));
            dump_state(static_cast<std::uint32_t>(pass));
        }
        std::printf("{\"leaves\": %zu}\n", tree().size());
        return 0;
    }
};

// ------------------------------------------------------------ Euler
template <int DIM, std::size_t N, std::size_t H, unsigned Depth>
struct euler_harness
{
    using shape_t = std::conditional_t<
        DIM == 2,
        amr::containers::static_shape<N, N>,
        amr::containers::static_shape<N, N, N>>;
    using layout_t       = amr::containers::static_layout<shape_t>;
    using patch_index_t  = amr::ndt::morton::morton_id<Depth, unsigned(DIM)>;
    using patch_layout_t = amr::ndt::patches::patch_layout<layout_t, H>;
    using interp_t = amr::ndt::intergrid_operator::linear_interpolator<patch_layout_t>;
    using cell_t   = std::conditional_t<DIM == 2, amr::cell::EulerCell2D, amr::cell::EulerCell3D>;
    using tree_t   = amr::ndt::tree::ndtree<cell_t, patch_index_t, patch_layout_t, interp_t>;
    static constexpr std::array<double, DIM> lengths = [] {
        std::array<double, DIM> l{};
        for (auto& e : l) e = 1000.0;
        return l;
    }();
    using geometry_t = amr::ndt::solver::physics_system<patch_index_t, patch_layout_t, lengths>;
    using phys_t     = EulerPhysics<DIM>;
    using solver_t   = amr_solver<tree_t, geometry_t, phys_t, DIM>;
    using padded_t   = typename patch_layout_t::padded_layout_t;
    using status_t   = typename tree_t::refine_status_t;
    using fields_t   = typename phys_t::FieldTags;
    static constexpr std::size_t flat = patch_layout_t::flat_size();
    static constexpr int         NVAR = phys_t::NVAR;

    params const&            P;
    writer&                  W;
    solver_t                 solver;
    std::vector<std::int8_t> last_flags;

    euler_harness(params const& p, writer& w)
        : P(p), W(w),
          solver(static_cast<std::size_t>(p.integer("capacity", 20000)), p.num("gamma", 1.4), p.num("cfl", 0.3))
    {
    }

    auto tree() -> tree_t& { return solver.get_tree(); }

    void dump_state(std::uint32_t step)
    {
        auto&               t = tree();
        const std::uint64_t n = t.size();
        // patch-major, fields in tuple order within a patch
        W.header(TAG_STATE, step, 16 + n * NVAR * flat * 8);
        W.put(n * NVAR);
        W.put(static_cast<std::uint64_t>(flat));
        for (std::size_t i = 0; i != n; ++i)
        {
            [&]<std::size_t... Is>(std::index_sequence<Is...>)
            {
                (
                    [&]
                    {
                        auto const& p = t.template get_patch<std::tuple_element_t<Is, fields_t>>(i);
                        for (std::size_t c = 0; c != flat; ++c)
                        {
                            double v = p[static_cast<typename padded_t::index_t>(c)];
                            W.put(v);
                        }
                    }(),
                    ...);
            }(std::make_index_sequence<NVAR>{});
        }
    }

    // the benchmark's acoustic_wave_amr_criterion: max Rho over the padded patch
    auto max_rho_status(patch_index_t const& idx) -> status_t
    {
        const double rthr = P.num("rthr", 0.53);
        const double cthr = P.num("cthr", 0.49);
        const int    minl = static_cast<int>(P.integer("min_level", 1));
        const int    maxl = static_cast<int>(P.integer("max_level", 6));
        auto const&  p    = tree().template get_patch<amr::cell::Rho>(idx);
        double       m    = 0.0;
        for (std::size_t c = 0; c != flat; ++c) m = std::max(p[static_cast<typename padded_t::index_t>(c)], m);
        const int level = static_cast<int>(idx.level());
        if (level < maxl && m > rthr) return status_t::Refine;
        if (level > minl && m < cthr) return status_t::Coarsen;
        return status_t::Stable;
    }

    int run()
    {
        auto refine_all = [](patch_index_t const&) { return status_t::Refine; };
        for (long i = 0; i < P.integer("init_levels", 3); ++i)
        {
            tree().reconstruct_tree(refine_all);
            tree().halo_exchange_update();
        }
        const double rho_bg = P.num("rho_bg", 0.5), p_bg = P.num("p_bg", 1.0), amp = P.num("amp", 10.0);
        const double width_sq = P.num("width_sq", 0.01 * 1000.0 * 1000.0);
        auto         pulse    = [&](auto const& coords) -> amr::containers::static_vector<double, NVAR>
        {
            double r_sq = 0.0;
            for (int d = 0; d < DIM; ++d)
            {
                const double dx = coords[d] - 0.5 * 1000.0;
                r_sq += dx * dx;
            }
            const double perturbation = amp * std::exp(-r_sq / width_sq);
            amr::containers::static_vector<double, NVAR> prim;
            prim[0] = rho_bg + (perturbation * 0.2);
            for (int d = 0; d < DIM; ++d) prim[1 + d] = 0.0;
            prim[DIM + 1] = p_bg + perturbation;
            return prim;
        };
        solver.initialize(pulse);
        tree().halo_exchange_update();
        dump_tree_records<DIM>(tree(), W, 0);
        dump_state(0);
        const long   steps    = P.integer("steps", 60);
        const long   interval = P.integer("remesh", 10);
        const double tmax     = P.num("tmax", 1e300);
        long         done = 0, batch = 0;
        double       t = 0.0;
        while (done < steps && t < tmax)
        {
            const long k = std::min(interval, steps - done);
            solver.advance_batch_async(static_cast<std::size_t>(k), tmax - t);
            std::size_t executed = 0;
            t += solver.finish_advance_batch(&executed);
            done += static_cast<long>(executed);
            ++batch;
            last_flags.clear();
            auto recording = [&](patch_index_t const& idx) -> status_t
            {
                const auto st = max_rho_status(idx);
                last_flags.push_back(static_cast<std::int8_t>(st));
                return st;
            };
            tree().reconstruct_tree(recording);
            tree().halo_exchange_update();
            W.header(TAG_FLAGS, static_cast<std::uint32_t>(done), 8 + last_flags.size());
            W.put(static_cast<std::uint64_t>(last_flags.size()));
            W.bytes(last_flags.data(), last_flags.size());
            dump_tree_records<DIM>(tree(), W, static_cast<std::uint32_t>(done));
            if (P.integer("state_every", 0) > 0 && batch % P.integer("state_every", 0) == 0)
                dump_state(static_cast<std::uint32_t>(done));
            if (executed == 0) break;
        }
        dump_state(static_cast<std::uint32_t>(done));
        W.header(TAG_DT, static_cast<std::uint32_t>(done), 16);
        W.put(t);
        W.put(static_cast<std::uint64_t>(done));
        std::printf("{\"steps\": %ld, \"time\": %.17g, \"leaves\": %zu}\n", done, t, tree().size());
        return 0;
    }
};

template <int DIM, std::size_t N, std::size_t H, unsigned Depth>
int dispatch(params const& p)
{
    writer w(p.str("out", "dump.bin"));
    const auto mode = p.str("mode", "run");
    if (mode == "euler")
    {
        auto      e  = std::make_unique<euler_harness<DIM, N, H, Depth>>(p, w);
        const int rc = e->run();
        if (rc == 0 && p.has("vtk"))
        {
            using geometry_t = typename euler_harness<DIM, N, H, Depth>::geometry_t;
            amr::ndt::print::vtk_print<geometry_t> printer(p.str("vtk", "tree"));
            printer.print(e->tree(), ".vtk");
        }
        return rc;
    }
    auto h = std::make_unique<harness<DIM, N, H, Depth>>(p, w);
    const int  rc   = mode == "tree" ? h->tree_mode() : (mode == "ssprk" ? h->ssprk_mode() : h->run());
    if (rc == 0 && p.has("vtk"))
    {
        using geometry_t = typename harness<DIM, N, H, Depth>::geometry_t;
        amr::ndt::print::vtk_print<geometry_t> printer(p.str("vtk", "tree"));
        printer.print(h->tree(), ".vtk");
    }
    return rc;
}

} // namespace harness

int main(int argc, char** argv)
{
    harness::params p;
    for (int i = 1; i < argc; ++i)
    {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) continue;
        p.kv[std::string(argv[i], static_cast<std::size_t>(eq - argv[i]))] = std::string(eq + 1);
    }
    const auto cfg = p.str("cfg", "2d16h1");
    if (cfg == "2d8h1") return harness::dispatch<2, 8, 1, 7>(p);
    if (cfg == "2d16h1") return harness::dispatch<2, 16, 1, 7>(p);
    if (cfg == "2d4h1") return harness::dispatch<2, 4, 1, 7>(p);
    if (cfg == "2d10h2") return harness::dispatch<2, 10, 2, 7>(p);
    if (cfg == "2d50h2") return harness::dispatch<2, 50, 2, 7>(p);
    if (cfg == "3d8h1") return harness::dispatch<3, 8, 1, 7>(p);
    if (cfg == "3d4h1") return harness::dispatch<3, 4, 1, 7>(p);
    std::fprintf(stderr, "unknown cfg %s\n", cfg.c_str());
    return 2;
}
