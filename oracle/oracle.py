"""ORACLE — test infrastructure, not the product.

ctypes binding of the C restatement of the gpu-amr reference (amr_oracle.c).
Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
load this module; the CUDA path never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

NEIGHBOR_DTYPE = np.dtype(
    [("kind", "u1"), ("quadrant", "u1", (3,)), ("pad", "<u4"), ("ids", "<u8", (4,))]
)

_lib = None


def build() -> Path:
    """Compile liboracle.so with the recipe in oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        vp, sz, u64, i32, dbl = C.c_void_p, C.c_size_t, C.c_uint64, C.c_int, C.c_double
        P = np.ctypeslib.ndpointer
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [i32, i32, i32, i32, sz]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_size.restype = sz
        L.oracle_size.argtypes = [vp]
        L.oracle_flat.restype = sz
        L.oracle_flat.argtypes = [vp]
        L.oracle_get_ids.argtypes = [vp, P(np.uint64, flags="C")]
        L.oracle_get_neighbors.argtypes = [vp, P(NEIGHBOR_DTYPE, flags="C")]
        L.oracle_get_state.argtypes = [vp, P(np.float64, flags="C")]
        L.oracle_set_state.argtypes = [vp, P(np.float64, flags="C")]
        L.oracle_reconstruct.restype = i32
        L.oracle_reconstruct.argtypes = [vp, P(np.int8, flags="C")]
        L.oracle_refine_all.argtypes = [vp, i32]
        L.oracle_halo_exchange.argtypes = [vp]
        L.oracle_flags_gradient.argtypes = [vp, dbl, dbl, i32, i32, P(np.int8, flags="C")]
        L.oracle_flags_max.argtypes = [vp, dbl, dbl, i32, i32, P(np.int8, flags="C")]
        L.oracle_flags_random.argtypes = [vp, u64, u64, dbl, dbl, i32, i32, P(np.int8, flags="C")]
        L.oracle_init_state.argtypes = [vp, P(np.float64, flags="C"), i32, dbl, u64]
        L.oracle_random_state.argtypes = [vp, u64]
        L.oracle_compute_dt.restype = dbl
        L.oracle_compute_dt.argtypes = [vp, P(np.float64, flags="C"), dbl]
        L.oracle_advance.restype = dbl
        L.oracle_advance.argtypes = [vp, sz, P(np.float64, flags="C"), dbl, dbl, C.POINTER(sz)]
        L.oracle_write_vtk.restype = C.c_int
        L.oracle_write_vtk.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.oracle_adjoint.restype = sz
        L.oracle_adjoint.argtypes = [vp, sz, P(np.float64, flags="C"), dbl, dbl, P(np.float64, flags="C"),
                                     P(np.float64, flags="C")]
        L.oracle_unit_hash.restype = dbl
        L.oracle_unit_hash.argtypes = [u64, u64, u64]
        L.oracle_encode.restype = u64
        L.oracle_encode.argtypes = [i32, i32, P(np.uint32, flags="C"), i32]
        L.oracle_decode.argtypes = [i32, u64, P(np.uint32, flags="C"), C.POINTER(i32)]
        L.oracle_child_of.restype = u64
        L.oracle_child_of.argtypes = [i32, i32, u64, i32]
        L.oracle_parent_of.restype = u64
        L.oracle_parent_of.argtypes = [i32, i32, u64]
        L.oracle_set_threads.argtypes = [i32]
        L.oracle_create_fields.restype = vp
        L.oracle_create_fields.argtypes = [i32, i32, i32, i32, sz, i32]
        L.oracle_nvar.restype = i32
        L.oracle_nvar.argtypes = [vp]
        L.oracle_set_lengths.argtypes = [vp, P(np.float64, flags="C")]
        L.oracle_euler_dt.restype = dbl
        L.oracle_euler_dt.argtypes = [vp, dbl, dbl]
        L.oracle_ssprk_advance.restype = dbl
        L.oracle_ssprk_advance.argtypes = [vp, sz, C.c_int, P(np.float64, flags="C"), dbl, dbl, C.POINTER(sz)]
        L.oracle_euler_advance.restype = dbl
        L.oracle_euler_advance.argtypes = [vp, sz, dbl, dbl, dbl, C.POINTER(sz), vp]
        L.oracle_euler_init_pulse.argtypes = [vp, dbl, dbl, dbl, dbl, dbl, P(np.float64, flags="C")]
        _lib = L
    return _lib


class OracleTree:
    """CPU restatement of ``ndtree`` + ``amr_solver`` for one scalar field."""

    def __init__(self, rank: int, n: int, halo: int = 1, depth: int = 7, capacity: int = 20000, nvar: int = 1,
                 lengths=None):
        """nvar > 1: that many fields per cell (Euler: rank + 2); lengths:
        domain lengths per Morton axis (default 1)."""
        self.rank, self.n, self.halo, self.depth, self.nvar = rank, n, halo, depth, nvar
        self._t = lib().oracle_create_fields(rank, n, halo, depth, capacity, nvar)
        if not self._t:
            raise ValueError("bad oracle tree parameters")
        self.pad1 = n + 2 * halo
        if lengths is not None:
            lib().oracle_set_lengths(self._t, np.ascontiguousarray(lengths, np.float64))

    def __del__(self):
        t = getattr(self, "_t", None)
        if t:
            lib().oracle_destroy(t)
            self._t = None

    @property
    def size(self) -> int:
        return lib().oracle_size(self._t)

    @property
    def flat(self) -> int:
        return lib().oracle_flat(self._t)

    def ids(self) -> np.ndarray:
        out = np.empty(self.size, np.uint64)
        lib().oracle_get_ids(self._t, out)
        return out

    def neighbors(self) -> np.ndarray:
        out = np.zeros(self.size * 2 * self.rank, NEIGHBOR_DTYPE)
        lib().oracle_get_neighbors(self._t, out)
        return out.reshape(self.size, 2 * self.rank)

    def state(self) -> np.ndarray:
        """(size, pad1, ...) for one field, (size, nvar, pad1, ...) for several."""
        out = np.empty(self.size * self.flat * self.nvar, np.float64)
        lib().oracle_get_state(self._t, out)
        if self.nvar == 1:
            return out.reshape((self.size,) + (self.pad1,) * self.rank)
        return out.reshape((self.size, self.nvar) + (self.pad1,) * self.rank)

    def set_state(self, s: np.ndarray) -> None:
        s = np.ascontiguousarray(s, np.float64).reshape(-1)
        assert s.size == self.size * self.flat * self.nvar
        lib().oracle_set_state(self._t, s)

    # -------------------------------------------------------------- Euler
    def euler_init_pulse(self, gamma=1.4, rho_bg=0.5, p_bg=1.0, amplitude=10.0, width_sq=0.01 * 1000.0 * 1000.0,
                         centre=(500.0, 500.0, 500.0)):
        c = np.zeros(3)
        c[: len(centre)] = centre
        lib().oracle_euler_init_pulse(self._t, gamma, rho_bg, p_bg, amplitude, width_sq, c)

    def euler_dt(self, gamma, cfl) -> float:
        return lib().oracle_euler_dt(self._t, gamma, cfl)

    def euler_advance(self, steps, gamma, cfl, remaining=1.7976931348623157e308):
        """(simulated time, executed steps, step sizes)."""
        ex = C.c_size_t(0)
        dts = np.zeros(max(1, steps))
        acc = lib().oracle_euler_advance(self._t, steps, gamma, cfl, remaining, C.byref(ex),
                                         dts.ctypes.data_as(C.c_void_p))
        return acc, ex.value, dts[: ex.value]

    def ssprk_advance(self, steps, order, velocity, cfl, remaining=1.7976931348623157e308):
        """(simulated time, executed steps) of SSPRK2/3 steps of advection."""
        v = np.zeros(3)
        v[: len(velocity)] = velocity
        ex = C.c_size_t(0)
        acc = lib().oracle_ssprk_advance(self._t, steps, order, v, cfl, remaining, C.byref(ex))
        return acc, ex.value

    def reconstruct(self, flags: np.ndarray) -> int:
        f = np.ascontiguousarray(flags, np.int8)
        assert f.size == self.size
        return lib().oracle_reconstruct(self._t, f)

    def refine_all(self, levels: int) -> None:
        lib().oracle_refine_all(self._t, levels)

    def halo_exchange(self) -> None:
        lib().oracle_halo_exchange(self._t)

    def flags_gradient(self, rthr, cthr, min_level, max_level) -> np.ndarray:
        out = np.empty(self.size, np.int8)
        lib().oracle_flags_gradient(self._t, rthr, cthr, min_level, max_level, out)
        return out

    def flags_max(self, rthr, cthr, min_level, max_level) -> np.ndarray:
        out = np.empty(self.size, np.int8)
        lib().oracle_flags_max(self._t, rthr, cthr, min_level, max_level, out)
        return out

    def flags_random(self, seed, pass_, p_refine, p_coarsen, min_level, max_level) -> np.ndarray:
        out = np.empty(self.size, np.int8)
        lib().oracle_flags_random(self._t, seed, pass_, p_refine, p_coarsen, min_level, max_level, out)
        return out

    def init_state(self, bumps, noise=0.0, noise_seed=0) -> None:
        b = np.ascontiguousarray(np.asarray(bumps, np.float64).reshape(-1))
        nb = b.size // (self.rank + 2)
        if b.size == 0:
            b = np.zeros(1)
        lib().oracle_init_state(self._t, b, nb, noise, noise_seed)

    def random_state(self, seed) -> None:
        lib().oracle_random_state(self._t, seed)

    def compute_dt(self, velocity, cfl) -> float:
        v = np.zeros(3)
        v[: len(velocity)] = velocity
        return lib().oracle_compute_dt(self._t, v, cfl)

    def advance(self, steps, velocity, cfl, remaining=1.7976931348623157e308):
        v = np.zeros(3)
        v[: len(velocity)] = velocity
        ex = C.c_size_t(0)
        acc = lib().oracle_advance(self._t, steps, v, cfl, remaining, C.byref(ex))
        return acc, ex.value


    def write_vtk(self, path, field="Scalar"):
        if lib().oracle_write_vtk(self._t, str(path).encode(), field.encode()) != 0:
            raise OSError(f"cannot write {path}")

    def adjoint(self, steps, velocity, cfl, lam_T, remaining=1.7976931348623157e308):
        """Gradient of <lam_T, u_T> w.r.t. the interior of the current state
        for advance(steps, velocity, cfl, remaining) on the frozen mesh."""
        v = np.zeros(3)
        v[: len(velocity)] = velocity
        lt = np.ascontiguousarray(lam_T, np.float64).reshape(-1)
        out = np.zeros_like(lt)
        lib().oracle_adjoint(self._t, steps, v, cfl, remaining, lt, out)
        return out.reshape((self.size,) + (self.pad1,) * self.rank)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def unit_hash(a: int, b: int, c: int) -> float:
    return lib().oracle_unit_hash(a, b, c)


def run_scenario(rank, n, halo, depth, *, init_levels, steps, remesh, velocity, cfl, bumps,
                 noise=0.0, noise_seed=0, crit="none", rthr=0.05, cthr=0.01, min_level=1,
                 max_level=5, capacity=20000, record=False):
    """The reference benchmark loop (bench_fvm_solver_integration_active_amr.b.cpp:220-250):
    advance a batch of ``remesh`` steps, then reconstruct with the criterion and
    exchange halos.  Returns (tree, sum_dt, steps, cell_updates, records)."""
    t = OracleTree(rank, n, halo, depth, capacity)
    t.refine_all(init_levels)
    t.init_state(bumps, noise, noise_seed)
    t.halo_exchange()
    records = []
    done, sum_dt, cell_updates = 0, 0.0, 0
    while done < steps:
        k = min(remesh, steps - done) if remesh > 0 else steps - done
        leaves = t.size
        acc, ex = t.advance(k, velocity, cfl)
        sum_dt += acc
        done += ex
        cell_updates += ex * leaves * n**rank
        if remesh > 0 and crit != "none":
            if crit == "grad":
                f = t.flags_gradient(rthr, cthr, min_level, max_level)
            else:
                f = t.flags_max(rthr, cthr, min_level, max_level)
            rc = t.reconstruct(f)
            if rc != 0:
                raise RuntimeError(f"oracle reconstruct failed: {rc}")
            t.halo_exchange()
            if record:
                records.append((done, f, t.ids(), t.neighbors()))
        if ex == 0:
            break
    return t, sum_dt, done, cell_updates, records
