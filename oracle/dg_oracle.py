"""CPU restatement (numpy, FP64) of the reference's nodal DG patch solver on a
uniform periodic tree.  Test infrastructure only: it checks the CUDA DG path
and never runs inside it.

Reference (paths within the reference project):
  configuration  include/config/generated_config.hpp (order 2, 2D, 4 variables
                 per node, 4x4 cells per patch, one ghost cell, SSPRK2,
                 advection with velocity 1, Courant number 0.5)
  basis          include/dg_helpers/basis/gauss_legendre.hpp:16-35 (points and
                 weights on [0, 1]), lagrange.hpp:37-67 (L_i, L_i'),
                 polynomial.hpp:85-93 (face kernels)
  tables         include/dg_helpers/globals/kernels.hpp:15-73 (face kernels at
                 0 and 1, mass tensors w (x) w and their inverse, derivative
                 tensor D[i][j] = L_i'(x_j))
  flux           include/dg_helpers/equations/advection.hpp:19-35 (F_d = v u)
  RHS            include/dg_helpers/rhs.hpp:117-255 with volume.hpp:24-44 and
                 surface.hpp:36-113 (Rusanov flux, surface mass, lift)
  stages         include/dg_helpers/time_integration/time.hpp:134-168 (SSPRK2)
  step loop      include/dg_helpers/solver.hpp:109-244 (dt = initial dt for the
                 first step, then min(dt, 0.1 x cell edge / |v| ...))

Each elementwise operation is evaluated in the reference's order and
grouping, so results are bit-identical to the reference on the same inputs
(pinned against fixtures produced by running the reference itself,
tests/golden/make_dg_golden.py).

State layout: U[cy, cx, ix, iy, v] over the global cell grid of a uniform
level (C = 4 * 2^level cells per side, cy rows, cx columns), nodes ix (x) and
iy (y), variables v.
"""
import numpy as np

ORDER, DIM, NVAR, PATCH = 2, 2, 4, 4
COURANT = 0.5
VELOCITY = 1.0


def tables():
    """Basis tables of the order-2 tensor Lagrange basis at Gauss-Legendre
    points on [0, 1], computed with the reference's arithmetic."""
    pre_p = np.array([-0.5773502691896257, 0.5773502691896257])
    pre_w = np.array([1.0, 1.0])
    half = (1.0 - 0.0) / 2.0
    mid = (0.0 + 1.0) / 2.0
    p = mid + half * pre_p
    w = pre_w * half

    def lag(i, x):
        num, den = 1.0, 1.0
        for k in range(ORDER):
            if k == i:
                continue
            num *= (x - p[k])
            den *= (p[i] - p[k])
        return num / den

    def dlag(i, x):
        res = 0.0
        for j in range(ORDER):
            if j == i:
                continue
            term = 1.0 / (p[i] - p[j])
            for k in range(ORDER):
                if k in (i, j):
                    continue
                term *= (x - p[k]) / (p[i] - p[k])
            res += term
        return res

    kern = np.array([[lag(i, 0.0) for i in range(ORDER)], [lag(i, 1.0) for i in range(ORDER)]])
    D = np.array([[dlag(i, p[j]) for j in range(ORDER)] for i in range(ORDER)])
    mass = np.outer(w, w)
    inv_w = 1.0 / w
    inv_mass = np.outer(inv_w, inv_w)
    return dict(points=p, weights=w, kern=kern, D=D, mass=mass, inv_mass=inv_mass, smass=w.copy())


T = tables()


def initial_state(level, t=0.0):
    """Nodal initial values of the advection scenario (advection.hpp:69-86):
    v0 = sin(2 pi (x + y - 2t)), v1 = sin(2 pi (y - t)), v2 = v3 = 1 at each
    node position (cell centre + (node - 0.5) x cell size)."""
    C = PATCH << level
    cell = (1.0 / float(1 << level)) / float(PATCH)
    U = np.empty((C, C, ORDER, ORDER, NVAR))
    cidx = np.arange(C, dtype=np.float64)
    # cell centres: patch corner + (local + 0.5) * cell; uniform grid gives
    # the same value as (global index + 0.5) * cell only up to rounding, so
    # follow the reference's corner + local form
    for cy in range(C):
        for cx in range(C):
            pcx, lcx = divmod(cx, PATCH)
            pcy, lcy = divmod(cy, PATCH)
            corner_x = float(pcx << (6 - level)) * (1.0 / float(1 << 6))
            corner_y = float(pcy << (6 - level)) * (1.0 / float(1 << 6))
            ccx = corner_x + (float(lcx) + 0.5) * cell
            ccy = corner_y + (float(lcy) + 0.5) * cell
            for ix in range(ORDER):
                for iy in range(ORDER):
                    x = ccx + (T["points"][ix] - 0.5) * cell
                    y = ccy + (T["points"][iy] - 0.5) * cell
                    U[cy, cx, ix, iy, 0] = np.sin(2.0 * 3.14159265358979323846 * (x + y - 2.0 * t))
                    U[cy, cx, ix, iy, 1] = np.sin(2.0 * 3.14159265358979323846 * (y - t))
                    U[cy, cx, ix, iy, 2:] = 1.0
    del cidx
    return U


GAMMA = 1.4  # the Euler equation's default heat capacity ratio (euler.hpp:38)


def euler_pressure(U):
    """compute_pressure (euler.hpp:69-82) per node: variables [mx, my, rho, E]."""
    rho, E = U[..., 2], U[..., 3]
    kin = 0.0
    for d in range(2):
        kin = kin + 0.5 * U[..., d] * U[..., d] / rho
    return (GAMMA - 1.0) * (E - kin)


def euler_flux(U):
    """evaluate_flux (euler.hpp:120-160): [F_x, F_y] per node."""
    rho, E = U[..., 2], U[..., 3]
    p = euler_pressure(U)
    out = []
    for dr in range(2):
        u = U[..., dr] / rho
        F = np.empty_like(U)
        for i in range(2):
            F[..., i] = U[..., i] * u
            if i == dr:
                F[..., i] = F[..., i] + p
        F[..., 2] = rho * u
        F[..., 3] = (E + p) * u
        out.append(F)
    return out


def euler_eig(U, normal):
    """max_eigenvalue (euler.hpp:165-181): from the cell's first node only,
    |u_n| + sqrt(gamma p / rho)."""
    U0 = U[..., 0, 0, :]
    rho = U0[..., 2]
    p = euler_pressure(U0)
    c = np.sqrt(GAMMA * p / rho)
    return np.abs(U0[..., normal] / rho) + c


def euler_initial_state(level):
    """EulerInitialCondition<2> (euler.hpp:227-253) at the nodes: pressure
    pulse exp(-100 r^2) + 1, rho 1, zero momentum."""
    C = PATCH << level
    cell = (1.0 / float(1 << level)) / float(PATCH)
    U = np.zeros((C, C, ORDER, ORDER, NVAR))
    for cy in range(C):
        for cx in range(C):
            pcx, lcx = divmod(cx, PATCH)
            pcy, lcy = divmod(cy, PATCH)
            ccx = float(pcx << (6 - level)) * (1.0 / float(1 << 6)) + (float(lcx) + 0.5) * cell
            ccy = float(pcy << (6 - level)) * (1.0 / float(1 << 6)) + (float(lcy) + 0.5) * cell
            for ix in range(ORDER):
                for iy in range(ORDER):
                    x = ccx + (T["points"][ix] - 0.5) * cell
                    y = ccy + (T["points"][iy] - 0.5) * cell
                    r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)
                    p = np.exp(-100.0 * r2) + 1.0
                    U[cy, cx, ix, iy, 2] = 1.0
                    U[cy, cx, ix, iy, 3] = p / (1.4 - 1.0)
    return U


def _contract(A, k, dim):
    """contract<dim>(A, k) (container_algorithms.hpp:217-298): the first term,
    then the second added (order 2)."""
    if dim == 0:
        return A[..., 0, :, :] * k[0] + A[..., 1, :, :] * k[1]
    return A[..., :, 0, :] * k[0] + A[..., :, 1, :] * k[1]


def _patch_running_max(e):
    """Running maximum of the local face speeds over a patch in the
    reference's loop order (cells row-major, faces in direction order;
    rhs.hpp:186-243): e[cy, cx, face] -> lambda[cy, cx, face]."""
    C = e.shape[0]
    lam = np.empty_like(e)
    for py in range(0, C, PATCH):
        for px in range(0, C, PATCH):
            run = -np.inf
            for ly in range(PATCH):
                for lx in range(PATCH):
                    for f in range(4):
                        v = e[py + ly, px + lx, f]
                        run = v if run < v else run  # std::max(run, v)
                        lam[py + ly, px + lx, f] = run
    return lam


FACES = ((0, -1), (0, 1), (1, -1), (1, 1))


def rhs(U, edge, equation="advection", lam_out=None):
    """Residual R(U) of every interior cell (rhs.hpp: volume, surface, inverse
    mass) on the periodic grid.  lam_out (list): receives each patch's final
    running maximum of the face speeds."""
    K, D, M = T["kern"], T["D"], T["mass"]
    vol = (1.0 * edge) * edge
    area = 1.0 * edge
    inv_jac = 1.0 / edge
    if equation == "advection":
        F = [VELOCITY * U, VELOCITY * U]
    else:
        F = euler_flux(U)
    s = inv_jac * vol
    du = np.zeros_like(U)
    # derivative_contraction(D, G, 0): r[i][j] = (0 + D[i,0] G[0][j]) + D[i,1] G[1][j]
    G = F[0] * M[None, None, :, :, None]  # tensor_dot(flux_x, volume_mass)
    c0 = np.empty_like(U)
    for i in range(ORDER):
        c0[:, :, i, :, :] = (0.0 + D[i, 0] * G[:, :, 0, :, :]) + D[i, 1] * G[:, :, 1, :, :]
    du = du + s * c0
    G = F[1] * M[None, None, :, :, None]
    c1 = np.empty_like(U)
    for j in range(ORDER):
        c1[:, :, :, j, :] = (0.0 + D[j, 0] * G[:, :, :, 0, :]) + D[j, 1] * G[:, :, :, 1, :]
    du = du + s * c1
    # face speeds: advection |v| = 1; Euler the running maximum over the patch
    # of max(eig(cell), eig(neighbour)) in the reference's loop order
    nbrs = []
    for pdim, sign in FACES:
        shift = (1, 0) if pdim == 0 else (0, 1)
        nbrs.append(np.roll(U, shift=(-sign * shift[0], -sign * shift[1]), axis=(0, 1)))
    if equation == "advection":
        lam = np.ones(U.shape[:2] + (4,))
    else:
        e = np.empty(U.shape[:2] + (4,))
        for f, (pdim, sign) in enumerate(FACES):
            adim = 1 - pdim
            a, b = euler_eig(U, adim), euler_eig(nbrs[f], adim)
            e[:, :, f] = np.where(a < b, b, a)  # std::max(eig(cell), eig(neighbour))
        lam = _patch_running_max(e)
    if lam_out is not None:
        lam_out.append(lam[PATCH - 1::PATCH, PATCH - 1::PATCH, 3])
    # faces in the reference's direction order: padded dimension 0 (y) -, +,
    # then dimension 1 (x) -, +; tensor dimension = 1 - padded dimension
    for f, (pdim, sign) in enumerate(FACES):
        adim = 1 - pdim
        sidx = 0 if sign < 0 else 1
        Un = nbrs[f]
        Fn = [VELOCITY * Un, VELOCITY * Un] if equation == "advection" else euler_flux(Un)
        uf = _contract(U, K[sidx], adim)
        ff = _contract(F[adim], K[sidx], adim)
        un = _contract(Un, K[1 - sidx], adim)
        fn = _contract(Fn[adim], K[1 - sidx], adim)
        lm = lam[:, :, f][:, :, None, None]
        nf = (float(sign) * (ff + fn) * 0.5 + (uf - un) * (0.5 * lm)) * area
        wf = nf * T["smass"][None, None, :, None]
        kv = K[sidx]
        if adim == 1:  # tensor_product(weighted, kernel): [face node][normal node]
            face = wf[:, :, :, None, :] * kv[None, None, None, :, None]
        else:          # tensor_product(kernel, weighted): [normal node][face node]
            face = kv[None, None, :, None, None] * wf[:, :, None, :, :]
        du = du - face
    return du * (T["inv_mass"] / vol)[None, None, :, :, None]


def ssprk2_step(U, edge, dt, equation="advection", lam_out=None):
    """One SSPRK2 step (time.hpp:134-168): u* = u + dt R(u);
    u' = ((u + u*) + dt R(u*)) * 0.5.  lam_out receives the second stage's
    per-patch speed maxima."""
    us = U + rhs(U, edge, equation) * dt
    return (U + us + rhs(us, edge, equation, lam_out) * dt) * 0.5


def run(level, steps, dt0=0.01, U=None, equation="advection"):
    """The reference's step loop on a uniform level without re-mesh: returns
    the states after each step and the step sizes used."""
    edge = (1.0 / float(1 << level)) / float(PATCH)
    if U is None:
        U = initial_state(level) if equation == "advection" else euler_initial_state(level)
    scale = 1.0 / (float(ORDER) ** DIM + 1.0)
    dt = dt0
    out, dts = [], []
    for _ in range(steps):
        lams = []
        U = ssprk2_step(U, edge, dt, equation, lams)
        out.append(U)
        dts.append(dt)
        dt_min = dt
        for lam in lams[0].ravel():  # per patch, in the tree's order (any order gives the minimum)
            if lam > 0.0:
                dt_min = min(dt_min, scale * COURANT * edge / lam)
        dt = min(dt, dt_min)
    return out, dts


# ---------------------------------------------------------------- layout
def morton_patch_order(level):
    """Patch (py, px) of each leaf of a uniform level in Morton order (x bits
    at even positions)."""
    n = 1 << level
    order = []
    for m in range(n * n):
        x = y = 0
        for b in range(level):
            x |= ((m >> (2 * b)) & 1) << b
            y |= ((m >> (2 * b + 1)) & 1) << b
        order.append((y, x))
    return order


def to_leaves(U, level):
    """Grid state -> leaves in Morton order, [leaf, cell (row-major, x
    fastest), node (ix * 2 + iy), variable]: the reference's dump layout."""
    P = PATCH
    out = []
    for (py, px) in morton_patch_order(level):
        blk = U[py * P:(py + 1) * P, px * P:(px + 1) * P]  # [ly, lx, ix, iy, v]
        out.append(blk.reshape(P * P, ORDER * ORDER, NVAR))
    return np.stack(out)


def from_leaves(L, level):
    P = PATCH
    C = P << level
    U = np.empty((C, C, ORDER, ORDER, NVAR))
    for n, (py, px) in enumerate(morton_patch_order(level)):
        U[py * P:(py + 1) * P, px * P:(px + 1) * P] = L[n].reshape(P, P, ORDER, ORDER, NVAR)
    return U


# ---------------------------------------------------------------- printer
MAX_DEPTH = 6  # morton_id<MaxDepth = 6, 2> of the DG tree (generated_config.hpp:32)


def _lagrange_quad_index(i, j, order):
    """point_idx_lagrange_quad (print_dg_tree_v2.hpp:61-97): VTK Lagrange
    quadrilateral point order (corners, edges, face)."""
    ib, jb = i in (0, order), j in (0, order)
    if ib and jb:
        return (2 if j > 0 else 1) if i > 0 else (3 if j > 0 else 0)
    if not ib and jb:
        return (i - 1) + (2 * (order - 1) if j > 0 else 0) + 4
    if ib and not jb:
        return (j - 1) + ((order - 1) if i > 0 else 3 * (order - 1)) + 4
    return 4 + 4 * (order - 1) + (i - 1) + (order - 1) * (j - 1)


def _decode(ids):
    """Patch origin of Morton ids (interleave << 6 | level) on the finest
    grid (2^MAX_DEPTH cells per axis): x from the even bits, y from the odd."""
    m = ids.astype(np.uint64) >> np.uint64(6)
    x = np.zeros(len(ids), np.int64)
    y = np.zeros(len(ids), np.int64)
    for b in range(MAX_DEPTH):
        x |= ((m >> np.uint64(2 * b)) & np.uint64(1)).astype(np.int64) << b
        y |= ((m >> np.uint64(2 * b + 1)) & np.uint64(1)).astype(np.int64) << b
    return x, y, (ids & np.uint64(63)).astype(np.int64)


def dg_vtk_bytes(ids, leaves):
    """dg_tree_printer_2d::print (print_dg_tree_v2.hpp:145-370) as bytes:
    every interior cell becomes a VTK Lagrange quadrilateral (type 70) with
    its polynomial (Basis::evaluate_basis, polynomial.hpp:36-55) evaluated at
    the (order + 1)^2 points xi, eta in {0, 1/2, 1}; legacy binary,
    big-endian.  ids: Morton ids in leaf order; leaves: [leaf, cell
    (row-major, x fastest), node (x-node * 2 + y-node), variable]."""
    T = tables()
    p = T["points"]
    lag = lambda i, x: (1.0 * (x - p[1 - i])) / (1.0 * (p[i] - p[1 - i]))  # Lagrange::evaluate
    P = len(ids)
    px, py, lv = _decode(np.asarray(ids, np.uint64))
    norm = float(1 << MAX_DEPTH)
    pts, vals, conn = [], [], []
    for n in range(P):
        csg = float(1 << (MAX_DEPTH - int(lv[n]))) / float(PATCH)
        for ly in range(PATCH):
            for lx in range(PATCH):
                cx = (float(px[n]) + (float(lx) + 0.5) * csg) / norm
                cy = (float(py[n]) + (float(ly) + 0.5) * csg) / norm
                h = csg / norm
                C = leaves[n, ly * PATCH + lx].reshape(ORDER, ORDER, NVAR)
                c = [0] * 9
                for jj in range(3):
                    for ii in range(3):
                        xi, eta = float(ii) / 2.0, float(jj) / 2.0
                        c[_lagrange_quad_index(ii, jj, 2)] = len(pts)
                        pts.append((cx + (2.0 * xi - 1.0) * (0.5 * h), cy + (2.0 * eta - 1.0) * (0.5 * h), 0.0))
                        s = np.zeros(NVAR)
                        for i0 in range(ORDER):
                            for i1 in range(ORDER):
                                prod = 1.0
                                prod *= lag(i0, xi)
                                prod *= lag(i1, eta)
                                s = s + C[i0, i1] * prod
                        vals.append(s)
                conn.append(c)
    out = [b"# vtk DataFile Version 3.0\nDG 2D Printer (Order=2)\nBINARY\nDATASET UNSTRUCTURED_GRID\n"]
    out.append(f"POINTS {len(pts)} double\n".encode())
    out.append(np.array(pts, ">f8").reshape(-1, 3).tobytes())
    ncell = len(conn)
    out.append(f"CELLS {ncell} {ncell * 10}\n".encode())
    cells = np.empty((ncell, 10), ">i4")
    cells[:, 0] = 9
    if ncell:
        cells[:, 1:] = np.array(conn)
    out.append(cells.tobytes())
    out.append(f"CELL_TYPES {ncell}\n".encode())
    out.append(np.full(ncell, 70, ">i4").tobytes())
    if pts:
        V = np.array(vals)
        out.append(f"POINT_DATA {len(pts)}\n".encode())
        for comp in range(NVAR):
            out.append(f"SCALARS dof_component_{comp} double 1\nLOOKUP_TABLE default\n".encode())
            out.append(V[:, comp].astype(">f8").tobytes())
    return b"".join(out)
