"""warp_reactor_gb300 -- GB300-native primordial-chemistry grid integrator.

Python host mirror of the reference reproducer's CUDA host path
(reproducer.cpp:7791-7975, ``run_cells_cuda``) over the C ABI in
``include/warp_reactor.h``.  The compute path is the CUDA library
``_build/libwarp_reactor.so`` (sm_103a); there is no CPU fallback: every entry
point raises if the library cannot be loaded.

Names follow the reference: a *cell* is one independent chemistry state
(``CollapseState``), ``completed_global_steps`` counts outer collapse steps, the
grid is ``grid_dim**3`` cells.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libwarp_reactor.so")

NUM_SPECIES = 14
NEQS = 15
MAX_COLLAPSE_STEPS = 1000
SPECIES = ("E", "Hp", "H", "Hm", "Dp", "D", "H2p", "Dm", "H2", "HDp", "HD", "HEpp", "HEp", "HE")

# IntegratorResult, reproducer.cpp:30-37
SUCCESS = 1
BAD_INPUTS = -1
DT_UNDERFLOW = -2
TOO_MANY_STEPS = -4
TOO_MUCH_ACCURACY_REQUESTED = -5
LU_DECOMPOSITION_ERROR = -7

MATH_PORTABLE = 0
MATH_CUDA = 1

POLICY_GRIDWIDE_INDEPENDENT = 0
POLICY_LEGACY_LOCAL = 1
POLICY_GRIDWIDE_CTA32 = 2

# CollapseState, reproducer.cpp:7455-7461 (216 bytes)
STATS_FIELDS = ("internal_steps", "rhs_calls", "jacobian_calls", "decompositions",
                "linear_solves", "accepted_steps", "rejected_steps")
COLLAPSE_STATE = np.dtype([
    ("rho", "<f8"), ("T", "<f8"), ("e", "<f8"), ("xn", "<f8", (NUM_SPECIES,)),
    ("time", "<f8"), ("density_driver", "<f8"), ("completed_steps", "<i4"), ("reserved_", "<i4"),
    ("stats", [(f, "<u8") for f in STATS_FIELDS]),
])
assert COLLAPSE_STATE.itemsize == 216

# PackedFinalState, reproducer.cpp:7488-7505 (172 bytes, packed)
PACKED_FINAL_STATE = np.dtype([
    ("cell", "<i4"), ("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("completed_steps", "<i4"),
    ("time", "<f8"), ("density_driver", "<f8"), ("rho", "<f8"), ("T", "<f8"), ("e", "<f8"),
    ("xn", "<f8", (NUM_SPECIES,)),
])
assert PACKED_FINAL_STATE.itemsize == 172


class RunTiming(ctypes.Structure):
    """wr_run_timing: device-time breakdown of the last wr_run."""
    _fields_ = [("run_ms", ctypes.c_double), ("prepare_ms", ctypes.c_double), ("advance_ms", ctypes.c_double),
                ("prepare_launches", ctypes.c_int32), ("advance_launches", ctypes.c_int32),
                ("outer_steps", ctypes.c_int32), ("reserved_", ctypes.c_int32)]


class WarpReactorError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with IntegratorResult {code}")
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run warp_reactor_gb300.build.build_all() "
                               "(the integrator has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.wr_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.wr_destroy.argtypes = [vp]
        L.wr_destroy.restype = None
        L.wr_upload.argtypes = [vp, vp]
        L.wr_download.argtypes = [vp, vp]
        L.wr_prepare.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, dp]
        L.wr_advance.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ip]
        L.wr_run.argtypes = [vp, ctypes.c_int, ip]
        L.wr_run_cells.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip]
        L.wr_make_collapse_state.argtypes = [vp]
        L.wr_make_collapse_state.restype = None
        L.wr_create_batch.argtypes = [ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.wr_grid_result.argtypes = [vp, ctypes.c_int, ip, ip]
        L.wr_grid_dt_history.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int]
        L.wr_make_batch_state.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, vp]
        L.wr_make_batch_state.restype = None
        L.wr_set_profiling.argtypes = [vp, ctypes.c_int]
        L.wr_set_advance_variant.argtypes = [vp, ctypes.c_int]
        L.wr_set_policy.argtypes = [vp, ctypes.c_int]
        L.wr_autotune.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip]
        L.wr_get_run_timing.argtypes = [vp, ctypes.POINTER(RunTiming)]
        L.wr_dt_history.argtypes = [vp, vp, ctypes.c_int]
        L.wr_diag_fp64_peak.argtypes = [dp]
        L.wr_diag_coop_phases.argtypes = [vp, ctypes.c_int]
        L.wr_diag_coop_phases_read.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
        L.wr_last_error.restype = ctypes.c_char_p
        L.wr_kernel_launch_count.restype = ctypes.c_uint64
        _lib = L
    return _lib


def last_error() -> str:
    return lib().wr_last_error().decode()


def kernel_launch_count() -> int:
    return int(lib().wr_kernel_launch_count())


def make_collapse_state() -> np.ndarray:
    """The reference's initial cell, ``make_collapse_state`` (reproducer.cpp:7543-7546)."""
    out = np.zeros(1, COLLAPSE_STATE)
    lib().wr_make_collapse_state(out.ctypes.data)
    return out[0]


def make_grid(grid_dim: int) -> np.ndarray:
    n = int(grid_dim) ** 3
    cells = np.empty(n, COLLAPSE_STATE)
    cells[:] = make_collapse_state()
    return cells


class Context:
    """Device state on one GPU (``wr_create`` .. ``wr_destroy``).

    ``Context(n)`` holds one grid of n cells.  ``Context(grids=[n0, n1, ...])``
    batches several independent grids (``wr_create_batch``): cells are
    concatenated grid after grid, each grid runs its own schedule, and one launch
    covers all of them.
    """

    def __init__(self, num_cells: int = 0, device: int = 0, math: int = MATH_CUDA, grids=None):
        h = ctypes.c_void_p()
        if grids is None:
            grids = [int(num_cells)]
        sizes = np.ascontiguousarray(np.asarray(grids, dtype=np.int32))
        rc = lib().wr_create_batch(len(sizes), sizes.ctypes.data, int(device), int(math), ctypes.byref(h))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_create ({last_error()})")
        self.handle = h
        self.grids = [int(v) for v in sizes]
        self.num_cells = int(sizes.sum())

    def close(self):
        if self.handle:
            lib().wr_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_cells(self, cells):
        if cells.dtype != COLLAPSE_STATE or cells.shape != (self.num_cells,) or not cells.flags.c_contiguous:
            raise ValueError("cells must be a contiguous COLLAPSE_STATE array of num_cells records")

    def upload(self, cells: np.ndarray) -> None:
        self._check_cells(cells)
        rc = lib().wr_upload(self.handle, cells.ctypes.data)
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_upload ({last_error()})")

    def download(self, cells: np.ndarray) -> None:
        self._check_cells(cells)
        rc = lib().wr_download(self.handle, cells.ctypes.data)
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_download ({last_error()})")

    def prepare(self, completed_global_steps: int, grid_time: float, step: int, perturb: bool):
        """prepare_grid_timestep_kernel + grid minimum -> (result, dt_grid)."""
        dt = ctypes.c_double()
        rc = lib().wr_prepare(self.handle, completed_global_steps, grid_time, step, int(bool(perturb)),
                              ctypes.byref(dt))
        return rc, dt.value

    def advance(self, completed_global_steps: int, next_grid_time: float, dt_grid: float):
        """advance_collapse_gridwide_kernel -> (result, integrated_count)."""
        cnt = ctypes.c_int()
        rc = lib().wr_advance(self.handle, completed_global_steps, next_grid_time, dt_grid, ctypes.byref(cnt))
        return rc, cnt.value

    def set_variant(self, variant: int) -> None:
        """Advance-kernel launch shape (0, 1, 2); results do not depend on it."""
        rc = lib().wr_set_advance_variant(self.handle, int(variant))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_set_advance_variant ({last_error()})")

    def set_policy(self, policy: int) -> None:
        """POLICY_GRIDWIDE_INDEPENDENT (default), POLICY_LEGACY_LOCAL or
        POLICY_GRIDWIDE_CTA32."""
        rc = lib().wr_set_policy(self.handle, int(policy))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_set_policy ({last_error()})")

    def autotune(self, perturb: bool = True, steps: int = 24) -> int:
        """Pick the fastest exact launch shape on the uploaded state; returns it."""
        best = ctypes.c_int(-1)
        rc = lib().wr_autotune(self.handle, int(bool(perturb)), int(steps), ctypes.byref(best))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_autotune ({last_error()})")
        return best.value

    def set_profiling(self, on: bool = True) -> None:
        rc = lib().wr_set_profiling(self.handle, int(bool(on)))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_set_profiling ({last_error()})")

    PHASES = ("queue_prologue_epilogue", "jacobian_rhs_program", "loads_gather_combinations", "lu", "stage_solves",
              "rhs_programs", "error_norm_controller")

    def phase_counters(self, on: bool = True) -> None:
        """Phase counters of the cooperative advance (wr_diag_coop_phases)."""
        rc = lib().wr_diag_coop_phases(self.handle, int(bool(on)))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_diag_coop_phases ({last_error()})")

    def read_phases(self, reset: bool = False) -> dict:
        """The phase counters: cycles per phase (summed over warps), attempts,
        total cycles and warps (wr_diag_coop_phases_read)."""
        buf = (ctypes.c_ulonglong * 16)()
        rc = lib().wr_diag_coop_phases_read(self.handle, buf, int(bool(reset)))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_diag_coop_phases_read ({last_error()})")
        out = {name: int(buf[k]) for k, name in enumerate(self.PHASES)}
        out.update({"attempts": int(buf[7]), "cycles": int(buf[8]), "warps": int(buf[9])})
        return out

    def run_timing(self) -> RunTiming:
        t = RunTiming()
        lib().wr_get_run_timing(self.handle, ctypes.byref(t))
        return t

    def dt_history(self, grid: int = 0) -> np.ndarray:
        out = np.zeros(MAX_COLLAPSE_STEPS)
        rc = lib().wr_grid_dt_history(self.handle, int(grid), out.ctypes.data, MAX_COLLAPSE_STEPS)
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_grid_dt_history ({last_error()})")
        return out

    def grid_result(self, grid: int):
        """(IntegratorResult, completed_global_steps) of one grid after run()."""
        cgs, res = ctypes.c_int(), ctypes.c_int()
        rc = lib().wr_grid_result(self.handle, int(grid), ctypes.byref(cgs), ctypes.byref(res))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_grid_result ({last_error()})")
        return res.value, cgs.value

    def run(self, perturb: bool = True, completed_global_steps: int = 0):
        """The whole outer loop on the device -> (result, completed_global_steps)."""
        cgs = ctypes.c_int(completed_global_steps)
        rc = lib().wr_run(self.handle, int(bool(perturb)), ctypes.byref(cgs))
        return rc, cgs.value


def run_cells(cells: np.ndarray, perturb: bool = True, math: int = MATH_CUDA, device: int = 0):
    """Mirror of ``run_cells_cuda(cells, perturb, completed_global_steps)``: advances
    ``cells`` in place and returns (IntegratorResult, completed_global_steps)."""
    with Context(len(cells), device, math) as ctx:
        ctx.upload(cells)
        rc, cgs = ctx.run(perturb)
        ctx.download(cells)
    return rc, cgs


def make_batch_grid(grid_id: int, num_cells: int, sigma_dex: float = 1.0, log10_tmin: float = 2.0,
                    log10_tmax: float = 4.0) -> np.ndarray:
    """Seeded cells of the batching workload (``wr_make_batch_state``): log-normal
    density (sigma in dex) and log-uniform temperature.  The temperature range
    starts at 100 K: below it the reference's analytic Jacobian evaluates to NaN
    (rate fits outside their range), and the reference integrator's reject loop
    never accepts a step."""
    out = np.zeros(int(num_cells), COLLAPSE_STATE)
    L = lib()
    for i in range(int(num_cells)):
        L.wr_make_batch_state(int(grid_id), i, sigma_dex, log10_tmin, log10_tmax, out[i:i + 1].ctypes.data)
    return out


def fp64_peak() -> float:
    """Measured FP64 FMA instructions per second of the current GPU."""
    v = ctypes.c_double()
    rc = lib().wr_diag_fp64_peak(ctypes.byref(v))
    if rc != SUCCESS:
        raise WarpReactorError(rc, "wr_diag_fp64_peak")
    return v.value


def pack_final_states(cells: np.ndarray, grid_dim: int) -> np.ndarray:
    """``make_packed_final_state`` for every cell (reproducer.cpp:8289-8305)."""
    n = len(cells)
    out = np.zeros(n, PACKED_FINAL_STATE)
    idx = np.arange(n, dtype=np.int64)
    out["cell"] = idx
    out["i"] = idx % grid_dim
    out["j"] = (idx // grid_dim) % grid_dim
    out["k"] = idx // (grid_dim * grid_dim)
    out["completed_steps"] = cells["completed_steps"]
    for f in ("time", "density_driver", "rho", "T", "e", "xn"):
        out[f] = cells[f]
    return out
