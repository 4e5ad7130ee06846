"""ORACLE -- test infrastructure only.

ctypes front end of the CPU oracle (``oracle/wr_oracle.cpp``) and, where it has
been built, of the reference itself (``oracle/_ref/libwr_ref.so``).  Only the
tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
module; the GPU library never does.

``load("port")``   oracle with the project's portable exp/log/cbrt (the GPU
                   library's default arithmetic)
``load("libm")``   oracle with the C library's exp/log/cbrt (the reference CPU
                   build's arithmetic)
``load("ref")``    the reference compiled from its own sources (only where the
                   reference tree was present at build time)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {
    "port": os.path.join(HERE, "_build", "libwr_oracle_port.so"),
    "libm": os.path.join(HERE, "_build", "libwr_oracle_libm.so"),
    "ref": os.path.join(HERE, "_ref", "libwr_ref.so"),
}

# same layout as warp_reactor_gb300.COLLAPSE_STATE (reproducer.cpp:7455-7461)
COLLAPSE_STATE = np.dtype([
    ("rho", "<f8"), ("T", "<f8"), ("e", "<f8"), ("xn", "<f8", (14,)),
    ("time", "<f8"), ("density_driver", "<f8"), ("completed_steps", "<i4"), ("reserved_", "<i4"),
    ("stats", [(f, "<u8") for f in ("internal_steps", "rhs_calls", "jacobian_calls", "decompositions",
                                    "linear_solves", "accepted_steps", "rejected_steps")]),
])

_cache = {}


def available(kind: str) -> bool:
    return os.path.exists(PATHS[kind])


class Oracle:
    def __init__(self, kind: str):
        path = PATHS[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built")
        self.kind = kind
        p = "wrr_" if kind == "ref" else "wro_"
        L = ctypes.CDLL(path)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C")
        vp = ctypes.c_void_p
        self._f = {}

        def fn(name, argtypes, restype=ctypes.c_int):
            f = getattr(L, p + name)
            f.argtypes = argtypes
            f.restype = restype
            self._f[name] = f

        fn("make_collapse_state", [vp], None)
        fn("rhs", [dp, dp], None)
        fn("jac", [dp, dp], None)
        fn("net_rhs", [dp, ctypes.c_double, dp], None)
        fn("net_jac", [dp, ctypes.c_double, dp, dp], None)
        fn("lu", [dp, ip])
        fn("lu_solve", [dp, ip, dp], None)
        fn("burn", [vp, ctypes.c_double])
        fn("prepare", [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                       ctypes.POINTER(ctypes.c_double), ctypes.c_int])
        fn("advance", [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                       ctypes.POINTER(ctypes.c_int), ctypes.c_int])
        fn("run", [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int])
        if kind != "ref":
            fn("run_legacy", [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                              ctypes.c_int])
            for name in ("exp", "log", "cbrt"):
                fn(name, [ctypes.c_double], ctypes.c_double)
        self.lib = L

    # ----------------------------------------------------------------- cells
    def make_collapse_state(self):
        out = np.zeros(1, COLLAPSE_STATE)
        self._f["make_collapse_state"](out.ctypes.data)
        return out[0]

    def make_grid(self, grid_dim: int):
        cells = np.empty(int(grid_dim) ** 3, COLLAPSE_STATE)
        cells[:] = self.make_collapse_state()
        return cells

    def run(self, cells, perturb=True, nthreads=None, max_steps=-1, completed_global_steps=0):
        """Host outer loop (reproducer.cpp:7856-7959) on ``cells`` in place."""
        assert cells.dtype == COLLAPSE_STATE and cells.flags.c_contiguous
        cgs = ctypes.c_int(completed_global_steps)
        rc = self._f["run"](cells.ctypes.data, len(cells), int(bool(perturb)), ctypes.byref(cgs),
                            int(max_steps), int(nthreads or os.cpu_count() or 1))
        return rc, cgs.value

    def run_legacy(self, cells, perturb=True, nthreads=None, max_steps=-1):
        """The reference CPU program's legacy-local loop (reproducer.cpp:8630-8648)."""
        assert cells.dtype == COLLAPSE_STATE and cells.flags.c_contiguous
        cgs = ctypes.c_int(0)
        rc = self._f["run_legacy"](cells.ctypes.data, len(cells), int(bool(perturb)), ctypes.byref(cgs),
                                   int(max_steps), int(nthreads or os.cpu_count() or 1))
        return rc, cgs.value

    def prepare(self, cells, cgs, grid_time, step, perturb=True, nthreads=None):
        dt = ctypes.c_double()
        rc = self._f["prepare"](cells.ctypes.data, len(cells), cgs, grid_time, step, int(bool(perturb)),
                                ctypes.byref(dt), int(nthreads or os.cpu_count() or 1))
        return rc, dt.value

    def advance(self, cells, cgs, next_grid_time, dt_grid, nthreads=None):
        cnt = ctypes.c_int()
        rc = self._f["advance"](cells.ctypes.data, len(cells), cgs, next_grid_time, dt_grid,
                                ctypes.byref(cnt), int(nthreads or os.cpu_count() or 1))
        return rc, cnt.value

    def burn(self, cell_array, dt):
        assert cell_array.dtype == COLLAPSE_STATE and len(cell_array) == 1
        return self._f["burn"](cell_array.ctypes.data, float(dt))

    # ----------------------------------------------------------------- network / LU
    def rhs(self, y):
        out = np.zeros(15)
        self._f["rhs"](np.ascontiguousarray(y, np.float64), out)
        return out

    def jac(self, y):
        out = np.zeros(225)
        self._f["jac"](np.ascontiguousarray(y, np.float64), out)
        return out.reshape(15, 15)

    def net_rhs(self, X, T):
        out = np.zeros(15)
        self._f["net_rhs"](np.ascontiguousarray(X, np.float64), float(T), out)
        return out

    def net_jac(self, X, T):
        J = np.zeros(225)
        f = np.zeros(15)
        self._f["net_jac"](np.ascontiguousarray(X, np.float64), float(T), J, f)
        return J.reshape(15, 15), f

    def lu(self, A):
        M = np.ascontiguousarray(A, np.float64).reshape(225).copy()
        ip = np.zeros(15, np.int32)
        info = self._f["lu"](M, ip)
        return info, M.reshape(15, 15), ip

    def lu_solve(self, LU, ip, b):
        x = np.ascontiguousarray(b, np.float64).copy()
        self._f["lu_solve"](np.ascontiguousarray(LU, np.float64).reshape(225), np.ascontiguousarray(ip, np.int32), x)
        return x

    def exp(self, x):
        return self._f["exp"](float(x))

    def log(self, x):
        return self._f["log"](float(x))

    def cbrt(self, x):
        return self._f["cbrt"](float(x))


def load(kind: str = "port") -> Oracle:
    if kind not in _cache:
        _cache[kind] = Oracle(kind)
    return _cache[kind]
