// Discrete adjoint of amr_solver's time integration on a frozen mesh, over
// the C ABI (amr_adjoint_*): the transposed flux update, halo fill and
// forward-Euler steps in reverse order, with a checkpoint (state and step
// sizes) every `checkpoint_every` steps.  No counterpart in the reference.
//
//   amr::gb300::adjoint adj(tree.handle(), 400, {1.0, 0.5, 0.0}, 0.4, 20);
//   adj.forward();                         // u_0 (tree state) -> u_T
//   adj.backward(d_lambda_T, d_lambda_0);  // d<lambda_T, u_T>/d u_0
#pragma once

#include <array>
#include <cstddef>
#include <limits>

#include "amr_gb300.h"
#include "ndtree/ndtree.hpp"

namespace amr::gb300 {

class adjoint {
public:
    adjoint(amr_tree* tree, std::size_t steps, const std::array<double, 3>& velocity, double cfl,
            std::size_t checkpoint_every = 20, double remaining_time = std::numeric_limits<double>::max())
    {
        check(amr_adjoint_create(tree, steps, velocity.data(), cfl, remaining_time, checkpoint_every, &m_h));
    }
    adjoint(const adjoint&)            = delete;
    adjoint& operator=(const adjoint&) = delete;
    ~adjoint() { amr_adjoint_destroy(m_h); }

    void forward() { check(amr_adjoint_forward(m_h)); }
    // device buffers of size() padded patches of the tree's dtype
    void backward(const void* lambda_T, void* lambda_0) { check(amr_adjoint_backward(m_h, lambda_T, lambda_0)); }
    // host buffers (copied through the adjoint's device buffers)
    void backward_host(const void* lambda_T, void* lambda_0)
    {
        check(amr_adjoint_backward_host(m_h, lambda_T, lambda_0));
    }
    void checkpoint(std::size_t index, void* dst) { check(amr_adjoint_checkpoint(m_h, index, dst)); }
    std::size_t checkpoints() const
    {
        std::size_t n = 0;
        check(amr_adjoint_checkpoint_count(m_h, &n));
        return n;
    }

private:
    amr_adjoint* m_h = nullptr;
};

} // namespace amr::gb300
