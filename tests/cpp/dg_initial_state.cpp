// DGSolver<Policy>::initial_state of the C++ DG drop-in on the CPU: reads
// Morton ids (uint64, native order) from the file named by the second
// argument and writes the initial state (fields x leaves x 6 x 6, float64)
// to the third; the first argument picks the equation ("advection" or
// "euler").  Only the host arithmetic runs: no device call.
#include "config/generated_config.hpp"
#include "dg_helpers/solver.hpp"

#include <cstdio>
#include <cstring>
#include <vector>

namespace
{
struct EulerPolicy : amr::config::GlobalConfigPolicy
{
    static constexpr amr::config::EquationType equation = amr::config::EquationType::Euler;
};

template <typename Policy>
int run(const char* in, const char* out)
{
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return 2;
    std::vector<uint64_t> ids;
    uint64_t              id = 0;
    while (std::fread(&id, sizeof id, 1, f) == 1) ids.push_back(id);
    std::fclose(f);
    const std::vector<double> state = amr::solver::DGSolver<Policy>::initial_state(ids);
    f                               = std::fopen(out, "wb");
    if (!f) return 2;
    std::fwrite(state.data(), sizeof(double), state.size(), f);
    std::fclose(f);
    return 0;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc < 4) return 2;
    if (std::strcmp(argv[1], "euler") == 0) return run<EulerPolicy>(argv[2], argv[3]);
    return run<amr::config::GlobalConfigPolicy>(argv[2], argv[3]);
}
