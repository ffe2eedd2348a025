"""Discrete adjoint of the frozen-mesh advection step, through the C ABI.

Bars (stated per test):
  * dot-product identity <lam_T, A u_0> = <A^T lam_T, u_0>: relative 1e-12
    (FP64), on 2:1 meshes with every neighbour relation, 2D and 3D;
  * GPU FP64 adjoint vs the oracle's independent scatter-form transpose:
    relative L2 <= 1e-12;
  * gradient of 0.5 ||u_T - u_target||^2 vs central finite differences
    (eps 1e-4) along seeded random directions: relative 1e-6 (FP64);
  * FP32 adjoint vs the FP64 oracle gradient: relative L2 <= 1e-5;
  * checkpoints equal the forward states bit for bit.
The torch.autograd.Function below exists for these checks only.
"""
import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _mesh(oracle_mod, amr, rank, n, h, seed, dtype, rounds=2):
    """An irregular 2:1 mesh built by the same random flag sequence in the
    oracle and on the GPU."""
    o = oracle_mod.OracleTree(rank, n, h, 6, 20000)
    t = amr.Tree(rank, n, h, 6, capacity=20000, dtype=dtype)
    o.refine_all(1)
    t.refine_uniform(1)
    for k in range(rounds):
        f = o.flags_random(seed, k + 1, 0.35, 0.3, 1, 4)
        assert o.reconstruct(f) == 0
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), o.ids())
    return o, t


def _interior_mask(shape, rank, n, h):
    m = np.zeros(shape, bool)
    m[(slice(None),) + (slice(h, n + h),) * rank] = True
    return m


def _gpu_adjoint(torch, amr, t, u0, lam_T, steps, vel, cfl, every):
    dt = torch.float64 if t.dtype == amr.F64 else torch.float32
    d_u0 = torch.from_numpy(np.ascontiguousarray(u0)).to("cuda", dt)
    t.load_state_device(d_u0.data_ptr(), t.size)
    adj = amr.Adjoint(t, steps, vel, cfl, every=every)
    adj.forward()
    uT = torch.empty_like(d_u0)
    t.download_state_device(uT.data_ptr(), t.size)
    lt = torch.from_numpy(np.ascontiguousarray(lam_T)).to("cuda", dt)
    l0 = torch.empty_like(lt)
    adj.backward(lt.data_ptr(), l0.data_ptr())
    return adj, uT.double().cpu().numpy(), l0.double().cpu().numpy()


CASES = [(2, 16, 1, (1.0, 0.5)), (2, 8, 1, (-0.7, 0.4)), (2, 6, 2, (0.3, -0.9)), (3, 4, 1, (0.6, -0.5, 0.8)),
         (2, 16, 1, (0.0, -1.0))]


@pytest.mark.parametrize("rank,n,h,vel", CASES)
def test_dot_product_and_oracle(amr, oracle_mod, torch_cuda, rank, n, h, vel):
    o, t = _mesh(oracle_mod, amr, rank, n, h, 21, amr.F64)
    rng = np.random.default_rng(3)
    o.set_state(rng.standard_normal((o.size,) + (o.pad1,) * rank))
    o.halo_exchange()
    u0 = o.state()
    lam_T = rng.standard_normal(u0.shape)
    steps = 13
    adj, uT, l0 = _gpu_adjoint(torch_cuda, amr, t, u0, lam_T, steps, vel, 0.4, every=5)
    m = _interior_mask(u0.shape, rank, n, h)
    lhs, rhs = np.sum(lam_T[m] * uT[m]), np.sum(l0[m] * u0[m])
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    assert not np.any(l0[~m])
    ref = o.adjoint(steps, vel, 0.4, lam_T)
    num = np.linalg.norm((l0 - ref)[m])
    assert num <= 1e-12 * np.linalg.norm(ref[m])


def test_checkpoints_are_forward_states(amr, oracle_mod, torch_cuda):
    torch = torch_cuda
    o, t = _mesh(oracle_mod, amr, 2, 16, 1, 5, amr.F64)
    o.random_state(4)
    o.halo_exchange()
    u0 = o.state()
    adj, uT, _ = _gpu_adjoint(torch, amr, t, u0, np.zeros_like(u0), 23, (0.8, 0.6), 0.4, every=5)
    assert adj.checkpoints == 6  # steps 0, 5, 10, 15, 20, 23
    buf = torch.empty(u0.shape, dtype=torch.float64, device="cuda")
    d_u0 = torch.from_numpy(u0).cuda()
    for i, step in enumerate([0, 5, 10, 15, 20, 23]):  # replay from u_0 on the same mesh
        t.load_state_device(d_u0.data_ptr(), t.size)
        if step:
            t.advance(step, (0.8, 0.6), 0.4)
            t.finish_advance()
        want = t.download_state()
        adj.checkpoint(i, buf.data_ptr())
        np.testing.assert_array_equal(interior(buf.cpu().numpy(), 2, 16, 1), interior(want, 2, 16, 1))


def test_remesh_invalidates_the_adjoint(amr, oracle_mod):
    _, t = _mesh(oracle_mod, amr, 2, 8, 1, 2, amr.F64)
    adj = amr.Adjoint(t, 4, (1.0, 0.0), 0.4, every=2)
    t.refine_uniform(1)
    with pytest.raises(amr.AmrError) as e:
        adj.forward()
    assert e.value.code == amr.AMR_ERR_INVALID


def _autograd(torch, amr):
    class Advect(torch.autograd.Function):
        """u_0 -> u_T (interior) through the C ABI; backward = the discrete
        adjoint.  Test-only wrapper."""

        @staticmethod
        def forward(ctx, u0, adj):
            t = adj.tree
            t.load_state_device(u0.contiguous().data_ptr(), t.size)
            adj.forward()
            uT = torch.empty_like(u0)
            t.download_state_device(uT.data_ptr(), t.size)
            ctx.adj = adj
            return uT

        @staticmethod
        def backward(ctx, g):
            l0 = torch.empty_like(g)
            ctx.adj.backward(g.contiguous().data_ptr(), l0.data_ptr())
            return l0, None

    return Advect.apply


def test_gradient_against_finite_differences_and_autograd(amr, oracle_mod, torch_cuda):
    """loss = 0.5 ||u_T - u_target||^2 over interior cells, u_target the
    solver's image of a seeded perturbation of u_0."""
    torch = torch_cuda
    rank, n, h, vel, steps = 2, 16, 1, (1.0, 0.5), 40
    o, t = _mesh(oracle_mod, amr, rank, n, h, 9, amr.F64)
    o.random_state(11)
    o.halo_exchange()
    u0 = torch.from_numpy(o.state()).cuda()
    mask = torch.from_numpy(_interior_mask(tuple(u0.shape), rank, n, h)).cuda()
    rng = np.random.default_rng(12)
    adj = amr.Adjoint(t, steps, vel, 0.4, every=8)
    advect = _autograd(torch, amr)
    with torch.no_grad():
        pert = u0 + 0.05 * torch.from_numpy(rng.standard_normal(tuple(u0.shape))).cuda() * mask
        target = advect(pert, adj)

    def loss_of(u):
        r = (advect(u, adj) - target) * mask
        return 0.5 * torch.sum(r * r)

    x = u0.clone().requires_grad_(True)
    L = loss_of(x)
    L.backward()
    grad = x.grad.detach()
    # the same gradient straight through the C ABI
    with torch.no_grad():
        r = ((advect(u0, adj) - target) * mask).contiguous()
        l0 = torch.empty_like(r)
        adj.backward(r.data_ptr(), l0.data_ptr())
    assert torch.equal(l0, grad)
    eps = 1e-4
    worst = 0.0
    for _ in range(8):
        v = torch.from_numpy(rng.standard_normal(tuple(u0.shape))).cuda() * mask
        with torch.no_grad():
            fd = (loss_of(u0 + eps * v) - loss_of(u0 - eps * v)) / (2 * eps)
        gv = torch.sum(grad * v)
        worst = max(worst, float(abs(fd - gv) / abs(gv)))
    assert worst <= 1e-6, worst
    # against the oracle's FP64 gradient
    ref = o.adjoint(steps, vel, 0.4, r.cpu().numpy())
    m = _interior_mask(ref.shape, rank, n, h)
    g = grad.cpu().numpy()
    assert np.linalg.norm((g - ref)[m]) <= 1e-12 * np.linalg.norm(ref[m])


def test_fp32_adjoint_against_fp64_oracle(amr, oracle_mod, torch_cuda):
    rank, n, h, vel, steps = 2, 16, 1, (-0.6, 0.9), 60
    o, t = _mesh(oracle_mod, amr, rank, n, h, 17, amr.F32)
    o.random_state(2)
    o.set_state(o.state().astype(np.float32).astype(np.float64))
    o.halo_exchange()
    u0 = o.state()
    lam_T = np.random.default_rng(8).standard_normal(u0.shape).astype(np.float32).astype(np.float64)
    _, _, l0 = _gpu_adjoint(torch_cuda, amr, t, u0, lam_T, steps, vel, 0.4, every=20)
    ref = o.adjoint(steps, vel, 0.4, lam_T)
    m = _interior_mask(u0.shape, rank, n, h)
    assert np.linalg.norm((l0 - ref)[m]) <= 1e-5 * np.linalg.norm(ref[m])


def test_forest_adjoint_dot_product(amr, torch_cuda):
    """Per-instance velocities: each instance's transpose is its own."""
    torch = torch_cuda
    K = 4
    f = amr.Tree(2, 8, 1, 5, capacity=4096, dtype=amr.F64, instances=K)
    f.refine_to_levels([1, 2, 3, 2])
    f.set_instance_params(velocity=[(1.0, 0.5), (-0.3, 0.8), (0.6, -0.6), (0.0, -1.0)])
    rng = np.random.default_rng(1)
    u0 = rng.standard_normal((f.size, 10, 10))
    lam_T = rng.standard_normal(u0.shape)
    adj, uT, l0 = _gpu_adjoint(torch, amr, f, u0, lam_T, 9, None, 0.4, every=4)
    m = _interior_mask(u0.shape, 2, 8, 1)
    lhs, rhs = np.sum(lam_T[m] * uT[m]), np.sum(l0[m] * u0[m])
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
