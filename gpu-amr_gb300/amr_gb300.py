"""Python binding of the GB300 AMR C ABI (include/amr_gb300.h) over ctypes.

The library must be the in-tree CUDA build (gpu-amr_gb300/lib/libamr_gb300.so);
there is no CPU fallback: every call raises if the library or a GPU is missing.

    tree = Tree(rank=2, n=16, halo=1, depth=7, capacity=20000)
    tree.refine_uniform(2)
    tree.upload_state(u)                 # (size, P1, P1) float64
    tree.advance(10, velocity=(1.0, 0.5), cfl=0.4)
    sum_dt, steps = tree.finish_advance()
    tree.flags_gradient(0.05, 0.01, 1, 5); tree.remesh()
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libamr_gb300.so"

AMR_OK, AMR_ERR_INVALID, AMR_ERR_CUDA, AMR_ERR_CAPACITY, AMR_ERR_UNBALANCED, AMR_ERR_UNSUPPORTED, AMR_ERR_NO_DEVICE = range(7)
F64, F32 = 0, 1
DG_ADVECTION, DG_EULER = 0, 1  # amr_tree_dg_set_equation

HALO_META = np.dtype(
    [("neighbor", "<i4"), ("finer_ids", "<i4", (4,)), ("quadrant", "<i4", (3,)), ("relation", "i1"), ("padding", "i1", (3,))]
)
assert HALO_META.itemsize == 36


class AmrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"amr status {code}: {msg}")
        self.code = code


class PatchGeometry(C.Structure):
    _fields_ = [("rank", C.c_int32), ("n", C.c_int32), ("halo", C.c_int32), ("depth", C.c_int32),
                ("lengths", C.c_double * 3)]


class TreeDesc(C.Structure):
    _fields_ = [("geom", PatchGeometry), ("capacity", C.c_size_t), ("dtype", C.c_int32), ("stream", C.c_void_p),
                ("instances", C.c_int32), ("fields", C.c_int32)]


class EulerParams(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("remesh_interval", C.c_uint64), ("gamma", C.c_double), ("cfl", C.c_double),
                ("end_time", C.c_double), ("refine_threshold", C.c_double), ("coarsen_threshold", C.c_double),
                ("min_level", C.c_int32), ("max_level", C.c_int32)]


class CycleParams(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("remesh_interval", C.c_uint64), ("velocity", C.c_double * 3),
                ("cfl", C.c_double), ("remaining_time", C.c_double), ("criterion", C.c_int32),
                ("min_level", C.c_int32), ("max_level", C.c_int32), ("options", C.c_int32),
                ("refine_threshold", C.c_double), ("coarsen_threshold", C.c_double)]


class CycleStats(C.Structure):
    _fields_ = [("executed_steps", C.c_uint64), ("sum_dt", C.c_double), ("cell_updates", C.c_uint64),
                ("remeshes", C.c_uint64), ("intervals", C.c_uint64), ("leaves_min", C.c_uint64),
                ("leaves_max", C.c_uint64), ("leaves_mean", C.c_double), ("persistent_intervals", C.c_uint64),
                ("graph_intervals", C.c_uint64), ("remeshes_changed", C.c_uint64)]


class DgStats(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("remeshes", C.c_uint64), ("cells", C.c_uint64),
                ("leaves_max", C.c_uint64), ("time", C.c_double), ("next_dt", C.c_double)]


CRITERIA = {"none": 0, "grad": 1, "gradient": 1, "max": 2}
RUN_PER_LAUNCH = 1
RUN_INSTANCE_PARAMS = 2
RUN_NO_GRAPH = 4
RUN_NO_FUSED = 8
RUN_FUSED = 16


class TransferTask(C.Structure):
    _fields_ = [("source_patch", C.c_int32), ("destination_patch", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(str(LIB_PATH))
        vp, sz, i32, dbl = C.c_void_p, C.c_size_t, C.c_int, C.c_double
        for name in ("amr_tree_create",):
            getattr(L, name).argtypes = [C.POINTER(TreeDesc), C.POINTER(vp)]
        L.amr_last_error.restype = C.c_char_p
        L.amr_launch_count.restype = C.c_uint64
        L.amr_tree_destroy.argtypes = [vp]
        L.amr_tree_size.argtypes = [vp, C.POINTER(sz)]
        L.amr_tree_patch_cells.argtypes = [vp, C.POINTER(sz)]
        L.amr_tree_upload_state.argtypes = [vp, vp, sz]
        L.amr_tree_download_state.argtypes = [vp, vp, sz]
        L.amr_tree_load_state_device.argtypes = [vp, vp, sz]
        L.amr_tree_download_state_device.argtypes = [vp, vp, sz]
        L.amr_tree_reset.argtypes = [vp]
        L.amr_tree_device_state.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
        L.amr_tree_get_ids.argtypes = [vp, vp, sz]
        L.amr_tree_get_levels.argtypes = [vp, vp, sz]
        L.amr_tree_get_neighbors.argtypes = [vp, vp, sz]
        L.amr_tree_halo_exchange.argtypes = [vp]
        L.amr_tree_flags_gradient.argtypes = [vp, dbl, dbl, i32, i32]
        L.amr_tree_flags_max.argtypes = [vp, dbl, dbl, i32, i32]
        L.amr_tree_set_flags.argtypes = [vp, vp, sz]
        L.amr_tree_get_flags.argtypes = [vp, vp, sz]
        L.amr_tree_remesh.argtypes = [vp, C.POINTER(i32)]
        L.amr_tree_refine_uniform.argtypes = [vp, i32]
        L.amr_tree_advance.argtypes = [vp, sz, C.POINTER(dbl), dbl, dbl]
        L.amr_tree_finish_advance.argtypes = [vp, C.POINTER(dbl), C.POINTER(sz)]
        L.amr_tree_synchronize.argtypes = [vp]
        L.amr_tree_run.argtypes = [vp, C.POINTER(CycleParams), C.POINTER(CycleStats)]
        L.amr_tree_set_timing.argtypes = [vp, i32]
        L.amr_tree_get_timing.argtypes = [vp, C.POINTER(dbl), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.amr_tree_set_instance_params.argtypes = [vp, vp, vp, sz]
        L.amr_tree_step_config.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.amr_selftest_wait_timeout.argtypes = [C.c_int32, C.POINTER(C.c_int32)]
        L.amr_tree_write_vtk.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.amr_tree_reserve.argtypes = [vp, sz]
        L.amr_tree_euler_advance.argtypes = [vp, sz, dbl, dbl, dbl]
        L.amr_tree_advance_ssprk.argtypes = [vp, sz, i32, C.POINTER(dbl), dbl, dbl]
        L.amr_tree_dg_advance.argtypes = [vp, sz, C.POINTER(dbl), C.POINTER(dbl)]
        L.amr_tree_dg_remesh.argtypes = [vp, dbl, dbl, C.POINTER(i32)]
        L.amr_tree_dg_run.argtypes = [vp, dbl, dbl, i32, dbl, dbl, C.POINTER(DgStats)]
        L.amr_tree_dg_set_equation.argtypes = [vp, i32]
        L.amr_tree_dg_write_vtk.argtypes = [vp, C.c_char_p]
        L.amr_tree_euler_run.argtypes = [vp, C.POINTER(EulerParams), C.POINTER(CycleStats)]
        L.amr_tree_capacity.argtypes = [vp, C.POINTER(sz)]
        L.amr_adjoint_create.argtypes = [vp, sz, vp, dbl, dbl, sz, C.POINTER(vp)]
        L.amr_adjoint_destroy.argtypes = [vp]
        L.amr_adjoint_forward.argtypes = [vp]
        L.amr_adjoint_backward.argtypes = [vp, vp, vp]
        L.amr_adjoint_checkpoint.argtypes = [vp, sz, vp]
        L.amr_adjoint_checkpoint_count.argtypes = [vp, C.POINTER(sz)]
        L.amr_tree_refine_to_levels.argtypes = [vp, vp, sz]
        L.amr_tree_instance_offsets.argtypes = [vp, vp, sz]
        L.amr_tree_instance_time.argtypes = [vp, vp, vp, sz]
        L.amr_halo_exchange_f64.argtypes = [vp, vp, sz, sz, C.POINTER(PatchGeometry), vp]
        L.amr_halo_exchange_f32.argtypes = [vp, vp, sz, sz, C.POINTER(PatchGeometry), vp]
        L.amr_interpolate_patches_f64.argtypes = [vp, vp, sz, C.POINTER(PatchGeometry), vp]
        L.amr_restrict_patches_f64.argtypes = [vp, vp, sz, C.POINTER(PatchGeometry), vp]
        L.amr_gather_patches.argtypes = [vp, vp, sz, vp, sz, vp]
        L.amr_compute_step_dt.argtypes = [vp, sz, C.POINTER(PatchGeometry), C.POINTER(dbl), dbl, vp, vp, vp, vp, vp]
        L.amr_time_step_f64.argtypes = [vp, vp, vp, sz, C.POINTER(PatchGeometry), C.POINTER(dbl), vp, vp]
        L.amr_flags_max_f64.argtypes = [vp, vp, sz, C.POINTER(PatchGeometry), dbl, dbl, i32, i32, vp, vp]
        _lib = L
    return _lib


def check(code):
    if code != AMR_OK:
        raise AmrError(code, lib().amr_last_error().decode())


def launch_count() -> int:
    return int(lib().amr_launch_count())


def geometry(rank, n, halo=1, depth=7, lengths=(1.0, 1.0, 1.0)) -> PatchGeometry:
    g = PatchGeometry()
    g.rank, g.n, g.halo, g.depth = rank, n, halo, depth
    for i in range(3):
        g.lengths[i] = lengths[i] if i < len(lengths) else 1.0
    return g


def _vec3(v):
    a = (C.c_double * 3)()
    for i, x in enumerate(list(v)[:3]):
        a[i] = float(x)
    return a


class Tree:
    """Device-resident ndtree + amr_solver state: one scalar field, or
    `fields` fields (the Euler cell: rho, rho u_d, E)."""

    def __init__(self, rank, n, halo=1, depth=7, capacity=20000, dtype=F64, lengths=(1.0, 1.0, 1.0), stream=None,
                 instances=1, fields=1):
        """instances > 1 makes a forest of independent trees (one root each).
        With fields > 1, host states are (fields, size, padded patch)."""
        self.rank, self.n, self.halo, self.depth = rank, n, halo, depth
        self.instances = int(instances)
        self.fields = int(fields)
        self.dtype = dtype
        self.np_dtype = np.float64 if dtype == F64 else np.float32
        self.pad1 = n + 2 * halo
        d = TreeDesc()
        d.geom = geometry(rank, n, halo, depth, lengths)
        d.capacity = capacity
        d.dtype = dtype
        d.stream = stream
        d.instances = self.instances
        d.fields = self.fields
        h = C.c_void_p()
        check(lib().amr_tree_create(C.byref(d), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().amr_tree_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def size(self) -> int:
        s = C.c_size_t()
        check(lib().amr_tree_size(self._h, C.byref(s)))
        return s.value

    @property
    def capacity(self) -> int:
        s = C.c_size_t()
        check(lib().amr_tree_capacity(self._h, C.byref(s)))
        return s.value

    def reserve(self, capacity):
        """Change the capacity, keeping leaves, state, tables and flags."""
        check(lib().amr_tree_reserve(self._h, capacity))

    @property
    def flat(self) -> int:
        s = C.c_size_t()
        check(lib().amr_tree_patch_cells(self._h, C.byref(s)))
        return s.value

    def upload_state(self, state):
        a = np.ascontiguousarray(state, self.np_dtype)
        if a.size % (self.flat * self.fields):
            raise AmrError(AMR_ERR_INVALID, "state is not a whole number of patches")
        check(lib().amr_tree_upload_state(self._h, a.ctypes.data, a.size // (self.flat * self.fields)))

    def download_state(self):
        lead = (self.fields, self.size) if self.fields > 1 else (self.size,)
        out = np.empty(lead + (self.pad1,) * self.rank, self.np_dtype)
        check(lib().amr_tree_download_state(self._h, out.ctypes.data, self.size))
        return out

    def load_state_device(self, ptr, num_patches):
        check(lib().amr_tree_load_state_device(self._h, C.c_void_p(ptr), num_patches))

    def download_state_device(self, ptr, num_patches):
        check(lib().amr_tree_download_state_device(self._h, C.c_void_p(ptr), num_patches))

    def reset(self):
        check(lib().amr_tree_reset(self._h))

    def device_state(self):
        cur, nxt = C.c_void_p(), C.c_void_p()
        check(lib().amr_tree_device_state(self._h, C.byref(cur), C.byref(nxt)))
        return cur.value, nxt.value

    def ids(self):
        out = np.empty(self.size, np.uint64)
        check(lib().amr_tree_get_ids(self._h, out.ctypes.data, self.size))
        return out

    def levels(self):
        out = np.empty(self.size, np.int32)
        check(lib().amr_tree_get_levels(self._h, out.ctypes.data, self.size))
        return out

    def neighbors(self):
        out = np.zeros(self.size * 2 * self.rank, HALO_META)
        check(lib().amr_tree_get_neighbors(self._h, out.ctypes.data, self.size))
        return out.reshape(self.size, 2 * self.rank)

    def halo_exchange(self):
        check(lib().amr_tree_halo_exchange(self._h))

    def flags_gradient(self, rthr, cthr, min_level, max_level):
        check(lib().amr_tree_flags_gradient(self._h, rthr, cthr, min_level, max_level))

    def flags_max(self, rthr, cthr, min_level, max_level):
        check(lib().amr_tree_flags_max(self._h, rthr, cthr, min_level, max_level))

    def set_flags(self, flags):
        f = np.ascontiguousarray(flags, np.int8)
        check(lib().amr_tree_set_flags(self._h, f.ctypes.data, f.size))

    def get_flags(self):
        out = np.empty(self.size, np.int8)
        check(lib().amr_tree_get_flags(self._h, out.ctypes.data, self.size))
        return out

    def remesh(self) -> bool:
        ch = C.c_int(0)
        check(lib().amr_tree_remesh(self._h, C.byref(ch)))
        return bool(ch.value)

    def refine_uniform(self, levels):
        check(lib().amr_tree_refine_uniform(self._h, levels))

    def advance(self, steps, velocity, cfl, remaining=1.7976931348623157e308):
        """velocity None: the per-instance velocities of set_instance_params."""
        v = None if velocity is None else _vec3(velocity)
        check(lib().amr_tree_advance(self._h, steps, v, cfl, remaining))

    # ------------------------------------------------------------ forests
    def set_instance_params(self, velocity=None, level_bounds=None):
        """velocity: (K, rank or 3) per instance; level_bounds: (K, 2) min/max."""
        K = self.instances
        vp = bp = None
        if velocity is not None:
            v = np.zeros((K, 3), np.float64)
            a = np.asarray(velocity, np.float64).reshape(K, -1)
            v[:, : a.shape[1]] = a
            vp = v
        if level_bounds is not None:
            bp = np.ascontiguousarray(np.asarray(level_bounds, np.int32).reshape(K, 2))
        check(lib().amr_tree_set_instance_params(self._h, None if vp is None else vp.ctypes.data,
                                                 None if bp is None else bp.ctypes.data, K))

    def refine_to_levels(self, targets):
        t = np.ascontiguousarray(np.asarray(targets, np.int32).reshape(self.instances))
        check(lib().amr_tree_refine_to_levels(self._h, t.ctypes.data, self.instances))

    def instance_offsets(self):
        out = np.empty(self.instances + 1, np.uint64)
        check(lib().amr_tree_instance_offsets(self._h, out.ctypes.data, self.instances + 1))
        return out.astype(np.int64)

    def instance_time(self):
        acc = np.empty(self.instances, np.float64)
        cnt = np.empty(self.instances, np.uint32)
        check(lib().amr_tree_instance_time(self._h, acc.ctypes.data, cnt.ctypes.data, self.instances))
        return acc, cnt

    def finish_advance(self):
        acc, ex = C.c_double(), C.c_size_t()
        check(lib().amr_tree_finish_advance(self._h, C.byref(acc), C.byref(ex)))
        return acc.value, ex.value

    def run(self, steps, interval, velocity, cfl, criterion="grad", rthr=0.05, cthr=0.01, min_level=1,
            max_level=5, remaining=1.7976931348623157e308, per_launch=False, cluster=0, graph=True,
            instance_params=False, fused=None) -> dict:
        """The benchmark loop (advance `interval` steps, flag, re-mesh) for
        `steps` steps; returns the run statistics.  per_launch: never the
        cluster kernel; graph=False: host-driven intervals; instance_params:
        per-instance velocities (set_instance_params); fused: True / False
        forces the fused interval kernel on / off (None: the default)."""
        if velocity is None:
            velocity, instance_params = (0.0, 0.0, 0.0), True
        prm = CycleParams()
        prm.steps, prm.remesh_interval = steps, interval
        for i, v in enumerate(list(velocity)[:3]):
            prm.velocity[i] = float(v)
        prm.cfl, prm.remaining_time = cfl, remaining
        prm.criterion = CRITERIA[criterion]
        prm.min_level, prm.max_level = min_level, max_level
        prm.refine_threshold, prm.coarsen_threshold = rthr, cthr
        prm.options = ((RUN_PER_LAUNCH if per_launch else 0) | (0 if graph else RUN_NO_GRAPH)
                       | (RUN_INSTANCE_PARAMS if instance_params else 0)
                       | (0 if fused is None else (RUN_FUSED if fused else RUN_NO_FUSED))
                       | ((int(cluster) & 0xFF) << 8))
        st = CycleStats()
        check(lib().amr_tree_run(self._h, C.byref(prm), C.byref(st)))
        return {f: getattr(st, f) for f, _ in CycleStats._fields_}

    def advance_ssprk(self, steps, order, velocity, cfl, remaining=1.7976931348623157e308):
        """SSPRK2 (order 2) or SSPRK3 (order 3) steps of advection; velocity
        None: the per-instance velocities.  finish_advance() as for advance."""
        v = None if velocity is None else _vec3(velocity)
        check(lib().amr_tree_advance_ssprk(self._h, steps, order, v, cfl, remaining))

    # -------------------------------------------------------------- DG
    def dg_set_equation(self, equation):
        """DG_ADVECTION (default) or DG_EULER ("advection" / "euler")."""
        if isinstance(equation, str):
            equation = {"advection": DG_ADVECTION, "euler": DG_EULER}[equation]
        check(lib().amr_tree_dg_set_equation(self._h, equation))

    def dg_write_vtk(self, path):
        """The reference's DG printer (VTK Lagrange quadrilaterals, the
        cells' polynomials at 9 points each) for the current state."""
        check(lib().amr_tree_dg_write_vtk(self._h, str(path).encode()))

    def dg_advance(self, steps, dt, time=0.0):
        """Nodal DG steps (order 2, 2D, 16 fields): returns (next step size,
        time).  dt is the step size of the first step; as in the reference's
        loop, each step first takes dt = min(dt, dt_min) and then adds that
        updated dt to time."""
        d, t = C.c_double(dt), C.c_double(time)
        check(lib().amr_tree_dg_advance(self._h, steps, C.byref(d), C.byref(t)))
        return d.value, t.value

    def dg_run(self, initial_dt=0.01, end_time=1.0, amr_interval=20, refine_threshold=0.05,
               coarsen_threshold=0.01):
        """The DG solver's loop (steps and re-meshes) to end_time: a dict of
        steps, remeshes, cells (the reference's processed-cell count),
        leaves_max, time, next_dt."""
        st = DgStats()
        check(lib().amr_tree_dg_run(self._h, initial_dt, end_time, amr_interval, refine_threshold,
                                    coarsen_threshold, C.byref(st)))
        return {f: getattr(st, f) for f, _ in DgStats._fields_}

    def dg_remesh(self, refine_threshold=0.05, coarsen_threshold=0.01):
        """The DG solver's re-mesh (gradient indicator, polynomial
        prolongation / restriction): returns whether the tree changed."""
        ch = C.c_int32(0)
        check(lib().amr_tree_dg_remesh(self._h, refine_threshold, coarsen_threshold, C.byref(ch)))
        return bool(ch.value)

    # -------------------------------------------------------------- Euler
    def euler_advance(self, steps, gamma, cfl, remaining=1.7976931348623157e308):
        """advance_batch_async with EulerPhysics: `steps` CFL steps (clamped
        to `remaining`); finish_advance() gives (simulated time, steps)."""
        check(lib().amr_tree_euler_advance(self._h, steps, gamma, cfl, remaining))

    def euler_run(self, steps, interval, gamma, cfl, end_time, rthr, cthr, min_level, max_level) -> dict:
        """The reference's Euler benchmark loop (advance `interval` steps with
        the time left, max-Rho flags, re-mesh) until `steps` steps ran or the
        simulated time reaches end_time; returns the run statistics."""
        prm = EulerParams()
        prm.steps, prm.remesh_interval, prm.gamma, prm.cfl, prm.end_time = steps, interval, gamma, cfl, end_time
        prm.refine_threshold, prm.coarsen_threshold = rthr, cthr
        prm.min_level, prm.max_level = min_level, max_level
        st = CycleStats()
        check(lib().amr_tree_euler_run(self._h, C.byref(prm), C.byref(st)))
        return {f: getattr(st, f) for f, _ in CycleStats._fields_}

    def write_vtk(self, path, field="Scalar"):
        """vtk_print::print of the current leaves and state (legacy binary VTK);
        with several fields, `field` names them separated by commas."""
        check(lib().amr_tree_write_vtk(self._h, str(path).encode(), field.encode()))

    def step_config(self):
        """(warps per block, copy stages, blocks) of the last 2D update."""
        w, st, b = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().amr_tree_step_config(self._h, C.byref(w), C.byref(st), C.byref(b)))
        return w.value, st.value, b.value

    def set_timing(self, enabled: bool):
        check(lib().amr_tree_set_timing(self._h, int(enabled)))

    def get_timing(self):
        ms, n, cells = C.c_double(), C.c_uint64(), C.c_uint64()
        check(lib().amr_tree_get_timing(self._h, C.byref(ms), C.byref(n), C.byref(cells)))
        return ms.value, n.value, cells.value

    def synchronize(self):
        check(lib().amr_tree_synchronize(self._h))


class Adjoint:
    """Discrete adjoint of Tree.advance(steps, velocity, cfl, remaining) on
    the tree's current (frozen) mesh, with a checkpoint every `every` steps.

        adj = Adjoint(tree, 400, (1.0, 0.5), 0.4, every=20)
        adj.forward()                           # u_0 (tree state) -> u_T
        adj.backward(lam_T_ptr, lam_0_ptr)      # device pointers

    velocity None: the per-instance velocities of set_instance_params."""

    def __init__(self, tree, steps, velocity, cfl, remaining=1.7976931348623157e308, every=20):
        self.tree = tree
        h = C.c_void_p()
        v = None if velocity is None else _vec3(velocity)
        check(lib().amr_adjoint_create(tree._h, steps, v, cfl, remaining, every, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().amr_adjoint_destroy(self._h)
            self._h = None

    __del__ = close

    def forward(self):
        check(lib().amr_adjoint_forward(self._h))

    def backward(self, lam_T_ptr, lam_0_ptr):
        check(lib().amr_adjoint_backward(self._h, C.c_void_p(lam_T_ptr), C.c_void_p(lam_0_ptr)))

    def checkpoint(self, index, dst_ptr):
        check(lib().amr_adjoint_checkpoint(self._h, index, C.c_void_p(dst_ptr)))

    @property
    def checkpoints(self) -> int:
        n = C.c_size_t()
        check(lib().amr_adjoint_checkpoint_count(self._h, C.byref(n)))
        return n.value


# ------------------------------------------------------------ initial data
# Host-side helpers for amr_solver::initialize (amr_solver.hpp:105-145): cell
# centres of every interior cell from physics_system::cell_coord
# (physics_system.hpp:107-138) and a sum-of-Gaussians field with seeded
# SplitMix64 noise keyed by (seed, Morton id, interior cell index).

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(x):
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return x ^ (x >> np.uint64(31))


def unit_hash(a, b, c):
    """SplitMix64-based uniform in [0, 1) of three 64-bit keys."""
    a, b, c = (np.asarray(v, dtype=np.uint64) for v in (a, b, c))
    h = _mix64(a ^ _mix64(b ^ _mix64(c)))
    return (h >> np.uint64(11)).astype(np.float64) * 2.0**-53


def decode_ids(ids, rank, depth=None):
    """Morton ids -> (coords[P, rank] on the 2^depth grid, level[P]).  With
    `depth`, an instance prefix above the interleaved bits is dropped."""
    ids = np.asarray(ids, np.uint64)
    level = (ids & np.uint64(63)).astype(np.int64)
    m = ids >> np.uint64(6)
    if depth is not None and rank * depth < 58:
        m = m & np.uint64((1 << (rank * depth)) - 1)
    coords = np.zeros((ids.size, rank), np.int64)
    for b in range(64 // rank):
        for k in range(rank):
            bit = (m >> np.uint64(rank * b + k)) & np.uint64(1)
            coords[:, k] |= bit.astype(np.int64) << b
    return coords, level


def cell_centres(ids, rank, n, depth, lengths=(1.0, 1.0, 1.0)):
    """(P, n, ..., n, rank) physical centres of interior cells; axis k of the
    last dimension is Morton axis k (x, y, z); cell array axes follow the
    layout (dim 0 slowest)."""
    coords, level = decode_ids(ids, rank, depth)
    maxc = float(1 << depth)
    P = coords.shape[0]
    out = np.empty((P,) + (n,) * rank + (rank,))
    grid = np.indices((n,) * rank)
    for k in range(rank):
        L = float(lengths[k])
        origin = L * coords[:, k].astype(np.float64) / maxc
        cs = (L * (2.0 ** (depth - level)).astype(np.float64) / maxc) / float(n)
        data_cell = grid[rank - 1 - k].astype(np.float64)
        shape = (P,) + (1,) * rank
        co = origin.reshape(shape) + data_cell[None] * cs.reshape(shape)
        out[..., k] = co + 0.5 * cs.reshape(shape)
    return out


def gaussian_state(ids, rank, n, halo, depth, bumps, noise=0.0, noise_seed=0, lengths=(1.0, 1.0, 1.0)):
    """Padded state (P, n+2h, ...) with sum_b a_b exp(-|x - c_b|^2 / (2 s_b^2))
    in the interior, plus noise * (2 U - 1); ghosts are zero."""
    x = cell_centres(ids, rank, n, depth, lengths)
    val = np.zeros(x.shape[:-1])
    b = np.asarray(bumps, np.float64).reshape(-1, rank + 2)
    for row in b:
        r2 = np.zeros(x.shape[:-1])
        for k in range(rank):
            diff = x[..., k] - row[k]
            r2 = r2 + diff * diff
        val = val + row[rank + 1] * np.exp(-r2 / (2.0 * row[rank] * row[rank]))
    if noise != 0.0:
        P = val.shape[0]
        cell = np.arange(n**rank, dtype=np.uint64).reshape((1,) + (n,) * rank)
        idv = np.asarray(ids, np.uint64).reshape((P,) + (1,) * rank)
        val = val + noise * (2.0 * unit_hash(np.uint64(noise_seed), idv, cell) - 1.0)
    P1 = n + 2 * halo
    out = np.zeros((val.shape[0],) + (P1,) * rank)
    out[(slice(None),) + (slice(halo, n + halo),) * rank] = val
    return out


def seeded_bumps(rank, count, seed, sigma=(0.02, 0.06), amp=(0.5, 2.0), lo=0.15, hi=0.85):
    """Seeded Gaussian bump parameters: centre (rank), sigma, amplitude each."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        c = rng.uniform(lo, hi, size=rank)
        out.extend(list(c) + [rng.uniform(*sigma), rng.uniform(*amp)])
    return [float(round(v, 6)) for v in out]
