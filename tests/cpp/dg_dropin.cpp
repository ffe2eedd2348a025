// The C++ DG drop-in (gpu-amr_gb300/host/dg_helpers/solver.hpp) used the way
// the reference's DG example uses its solver: SimulationParams, a
// DGSolver<policy>, run().  The policy shortens the end time so that the run
// is brief.  Output: the VTK files under ./vtk_output, a line
// "processed <cells> files <n> leaves <P>" on stdout, and in the file named
// by the first argument two records, the tree after construction and after
// run(): leaf count (uint64), Morton ids (uint64 each), state (fields x
// leaves x 6 x 6, float64).
#include "config/generated_config.hpp"
#include "dg_helpers/solver.hpp"

#include <cstdio>
#include <filesystem>
#include <iostream>
#include <vector>

namespace
{
struct ShortPolicy : amr::config::GlobalConfigPolicy
{
    static constexpr double EndTime = 0.05;
};
} // namespace

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: dg_dropin <state file>\n";
        return 2;
    }
    try {
        amr::solver::SimulationParams params{
            .initial_dt    = 0.01,
            .plot_interval = 0.01,
            .initial_level = 5,
            .amr_interval  = 20,
        };
        amr::solver::DGSolver<ShortPolicy> solver(params);
        std::FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 2;
        std::size_t P      = 0;
        auto        record = [&]() {
            amr::solver::detail::dg_check(amr_tree_size(solver.tree(), &P));
            std::vector<uint64_t> ids(P);
            std::vector<double>   state(16 * P * 36);
            amr::solver::detail::dg_check(amr_tree_get_ids(solver.tree(), ids.data(), P));
            amr::solver::detail::dg_check(amr_tree_download_state(solver.tree(), state.data(), P));
            const uint64_t n = P;
            std::fwrite(&n, sizeof n, 1, f);
            std::fwrite(ids.data(), sizeof(uint64_t), P, f);
            std::fwrite(state.data(), sizeof(double), state.size(), f);
        };
        record();
        solver.run();
        record();
        std::fclose(f);

        std::size_t files = 0;
        for (const auto& e : std::filesystem::directory_iterator("vtk_output")) files += e.is_regular_file();
        std::cout << "processed " << solver.processed_cells() << " files " << files << " leaves " << P << "\n";
    } catch (const std::exception& e) {
        std::cerr << "Exception: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
