"""The oracle's adjoint (CPU, FP64) against the oracle's own forward: the
dot-product identity <lam_T, A u_0> = <A^T lam_T, u_0> on 2:1 meshes with
every neighbour relation, 2D and 3D, ghost layers 1 and 2 (relative 1e-13)."""
import numpy as np
import pytest


@pytest.mark.parametrize("rank,n,h,vel", [(2, 8, 1, (0.7, -0.4)), (2, 16, 1, (-1.0, 0.5)), (2, 6, 2, (0.3, 0.9)),
                                          (3, 4, 1, (0.6, -0.5, 0.8))])
def test_oracle_adjoint_dot_product(oracle_mod, rank, n, h, vel):
    t = oracle_mod.OracleTree(rank, n, h, 6, 20000)
    t.refine_all(1)
    for k in range(2):
        assert t.reconstruct(t.flags_random(5, k + 1, 0.3, 0.4, 1, 4)) == 0
    rng = np.random.default_rng(1)
    t.set_state(rng.standard_normal((t.size,) + (t.pad1,) * rank))
    t.halo_exchange()
    u0 = t.state()
    lam_T = rng.standard_normal(u0.shape)
    lam_0 = t.adjoint(7, vel, 0.4, lam_T)
    t.advance(7, vel, 0.4)
    uT = t.state()
    sl = (slice(None),) + (slice(h, n + h),) * rank
    lhs, rhs = np.sum(lam_T[sl] * uT[sl]), np.sum(lam_0[sl] * u0[sl])
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)
    g = lam_0.copy()
    g[sl] = 0.0
    assert not g.any()
