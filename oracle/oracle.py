"""ORACLE -- test infrastructure only.

ctypes front end of the CPU oracle (``oracle/wr_oracle.cpp``) and, where it has
been built, of the reference itself (``oracle/_ref/libwr_ref.so``).  Only the
tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
module; the GPU library never does.

``load("port")``   oracle with the project's portable exp/log/cbrt (the GPU
                   library's default arithmetic)
``load("libm")``   oracle with the C library's exp/log/cbrt (the reference CPU
                   build's arithmetic)
``load("prec")``   the precision form's arithmetic (FP32 factorisation in
                   error-weighted variables, one FP64 residual sweep per stage
                   solve; portable exp/log), the checker of advance variant 3
``load("ref")``    the reference compiled from its own sources (only where the
                   reference tree was present at build time)
``load_diff()``    the differentiation form's map with a frozen controller and its
                   FP64 tangent-linear (``oracle/wr_oracle_diff.cpp``)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {
    "port": os.path.join(HERE, "_build", "libwr_oracle_port.so"),
    "libm": os.path.join(HERE, "_build", "libwr_oracle_libm.so"),
    "prec": os.path.join(HERE, "_build", "libwr_oracle_prec.so"),
    "ref": os.path.join(HERE, "_ref", "libwr_ref.so"),
    "diff": os.path.join(HERE, "_build", "libwr_oracle_diff.so"),
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
            fn("run_cta32", [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
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

    def run_cta32(self, cells, perturb=True, nthreads=None, max_steps=-1):
        """The gridwide-structured-cta32 policy: one ROS2S controller per 32-cell
        tile (structured_cuda.cuh:393-782) under the same outer loop."""
        assert cells.dtype == COLLAPSE_STATE and cells.flags.c_contiguous
        cgs = ctypes.c_int(0)
        rc = self._f["run_cta32"](cells.ctypes.data, len(cells), int(bool(perturb)), ctypes.byref(cgs),
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


class DiffOracle:
    """The differentiation form's discrete map on the CPU (see wr_oracle_diff.cpp).

    ``record`` runs the reference controller and returns the accepted step sizes
    (``hbuf``, n x cap) and per-outer-step counts (n x nsteps); ``replay`` runs the
    frozen map on them; ``tangent`` its FP64 tangent-linear.  Outputs ``q`` are
    n x 15: the final xn[0..13] and T of each cell."""

    def __init__(self):
        path = PATHS["diff"]
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built")
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        i32 = ctypes.c_int
        L.wro_diff_num_multipliers.restype = i32
        L.wro_diff_forward.argtypes = [vp, vp, i32, i32, vp, i32, vp, vp, i32, vp, i32, vp, vp, i32]
        L.wro_diff_forward.restype = i32
        L.wro_diff_tangent.argtypes = [vp, vp, i32, i32, vp, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp, i32]
        L.wro_diff_tangent.restype = i32
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        L.wro_netp_rhs.argtypes = [dp, ctypes.c_double, dp, dp]
        L.wro_netp_rhs.restype = None
        L.wro_netp_rhs_vjp.argtypes = [dp, ctypes.c_double, dp, dp, dp, dp, dp]
        L.wro_netp_rhs_vjp.restype = None
        L.wro_netp_rhs_jvp.argtypes = [dp, ctypes.c_double, dp, dp, ctypes.c_double, dp, dp, dp]
        L.wro_netp_rhs_jvp.restype = None
        L.wro_net_jac_vjp.argtypes = [dp, ctypes.c_double, dp, dp, dp]
        L.wro_net_jac_vjp.restype = None
        L.wro_net_jac_jvp.argtypes = [dp, ctypes.c_double, dp, ctypes.c_double, dp, dp]
        L.wro_net_jac_jvp.restype = None
        self.lib = L
        self.num_multipliers = L.wro_diff_num_multipliers()

    @staticmethod
    def _p(a):
        return None if a is None else a.ctypes.data

    # generated derivative code (raw network at (X, T), no flooring / EOS)
    def rhs(self, X, T, mult):
        f = np.zeros(15)
        self.lib.wro_netp_rhs(np.ascontiguousarray(X, np.float64), float(T), np.ascontiguousarray(mult, np.float64), f)
        return f

    def rhs_vjp(self, X, T, mult, fbar):
        Xb, Tb, mb = np.zeros(14), np.zeros(1), np.zeros(self.num_multipliers)
        self.lib.wro_netp_rhs_vjp(np.ascontiguousarray(X, np.float64), float(T), np.ascontiguousarray(mult, np.float64),
                                  np.ascontiguousarray(fbar, np.float64), Xb, Tb, mb)
        return Xb, Tb[0], mb

    def rhs_jvp(self, X, T, mult, dX, dT, dmult):
        f, df = np.zeros(15), np.zeros(15)
        self.lib.wro_netp_rhs_jvp(np.ascontiguousarray(X, np.float64), float(T), np.ascontiguousarray(mult, np.float64),
                                  np.ascontiguousarray(dX, np.float64), float(dT),
                                  np.ascontiguousarray(dmult, np.float64), f, df)
        return f, df

    def jac_vjp(self, X, T, Jbar):
        Xb, Tb = np.zeros(14), np.zeros(1)
        self.lib.wro_net_jac_vjp(np.ascontiguousarray(X, np.float64), float(T),
                                 np.ascontiguousarray(Jbar, np.float64).reshape(225), Xb, Tb)
        return Xb, Tb[0]

    def jac_jvp(self, X, T, dX, dT):
        J, dJ = np.zeros(225), np.zeros(225)
        self.lib.wro_net_jac_jvp(np.ascontiguousarray(X, np.float64), float(T), np.ascontiguousarray(dX, np.float64),
                                 float(dT), J, dJ)
        return J.reshape(15, 15), dJ.reshape(15, 15)

    def record(self, cells, dt_hist, perturb=True, u=None, log_mult=None, cell_ids=None, cap=65536,
               nthreads=None):
        n, nsteps = len(cells), len(dt_hist)
        cells = np.ascontiguousarray(cells)
        dt_hist = np.ascontiguousarray(dt_hist, np.float64)
        hbuf = np.zeros((n, cap))
        counts = np.zeros((n, nsteps), np.int32)
        q = np.zeros((n, 15))
        u = None if u is None else np.ascontiguousarray(u, np.float64)
        lm = None if log_mult is None else np.ascontiguousarray(log_mult, np.float64)
        ids = None if cell_ids is None else np.ascontiguousarray(cell_ids, np.int32)
        rc = self.lib.wro_diff_forward(cells.ctypes.data, self._p(ids), n, int(bool(perturb)),
                                       dt_hist.ctypes.data, nsteps, self._p(u), self._p(lm), 1,
                                       hbuf.ctypes.data, cap, counts.ctypes.data, q.ctypes.data,
                                       int(nthreads or os.cpu_count() or 1))
        return rc, q, hbuf, counts

    def replay(self, cells, dt_hist, hbuf, counts, perturb=True, u=None, log_mult=None, cell_ids=None,
               nthreads=None):
        n, nsteps = len(cells), len(dt_hist)
        cells = np.ascontiguousarray(cells)
        dt_hist = np.ascontiguousarray(dt_hist, np.float64)
        hbuf = np.ascontiguousarray(hbuf, np.float64)
        counts = np.ascontiguousarray(counts, np.int32).copy()
        q = np.zeros((n, 15))
        u = None if u is None else np.ascontiguousarray(u, np.float64)
        lm = None if log_mult is None else np.ascontiguousarray(log_mult, np.float64)
        ids = None if cell_ids is None else np.ascontiguousarray(cell_ids, np.int32)
        rc = self.lib.wro_diff_forward(cells.ctypes.data, self._p(ids), n, int(bool(perturb)),
                                       dt_hist.ctypes.data, nsteps, self._p(u), self._p(lm), 0,
                                       hbuf.ctypes.data, hbuf.shape[1], counts.ctypes.data, q.ctypes.data,
                                       int(nthreads or os.cpu_count() or 1))
        return rc, q

    def tangent(self, cells, dt_hist, hbuf, counts, du=None, dlog_mult=None, perturb=True, u=None,
                log_mult=None, cell_ids=None, nthreads=None):
        n, nsteps = len(cells), len(dt_hist)
        cells = np.ascontiguousarray(cells)
        dt_hist = np.ascontiguousarray(dt_hist, np.float64)
        hbuf = np.ascontiguousarray(hbuf, np.float64)
        counts = np.ascontiguousarray(counts, np.int32)
        q = np.zeros((n, 15))
        dq = np.zeros((n, 15))
        u = None if u is None else np.ascontiguousarray(u, np.float64)
        lm = None if log_mult is None else np.ascontiguousarray(log_mult, np.float64)
        du = None if du is None else np.ascontiguousarray(du, np.float64)
        dlm = None if dlog_mult is None else np.ascontiguousarray(dlog_mult, np.float64)
        ids = None if cell_ids is None else np.ascontiguousarray(cell_ids, np.int32)
        rc = self.lib.wro_diff_tangent(cells.ctypes.data, self._p(ids), n, int(bool(perturb)),
                                       dt_hist.ctypes.data, nsteps, self._p(u), self._p(lm), self._p(du),
                                       self._p(dlm), hbuf.ctypes.data, hbuf.shape[1], counts.ctypes.data,
                                       q.ctypes.data, dq.ctypes.data, int(nthreads or os.cpu_count() or 1))
        return rc, q, dq


def load_diff() -> DiffOracle:
    if "diff" not in _cache:
        _cache["diff"] = DiffOracle()
    return _cache["diff"]


def grid_schedule(oracle: Oracle, cells, perturb=True, nthreads=None):
    """Runs the gridwide host loop (reproducer.cpp:7856-7959) on ``cells`` in place
    and returns (rc, dt_grid of every outer step)."""
    hist = []
    cgs, grid_time = 0, 0.0
    rc = 1
    for step in range(1000):
        rc, dt = oracle.prepare(cells, cgs, grid_time, step, perturb, nthreads)
        if rc != 1 or dt == np.finfo(np.float64).max:
            break
        rc, cnt = oracle.advance(cells, cgs, grid_time + dt, dt, nthreads)
        if rc != 1 or cnt == 0:
            if rc == 1:
                hist.append(dt)
            break
        hist.append(dt)
        grid_time += dt
        cgs += 1
    return rc, np.array(hist)
