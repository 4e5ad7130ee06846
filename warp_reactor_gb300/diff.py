"""Differentiation form: gradients of a grid's final chemistry state.

Python front end of the C ABI in ``include/warp_reactor_diff.h`` (kernels in
``csrc/wr_diff*.cu``).  The map, for one grid of cells advanced by the
gridwide-independent policy through a fixed outer schedule (the reference's
prepare/advance kernels per cell, reproducer.cpp:7696-7785):

    q = F(u, p)
    u[n, 15]  per cell xn[0..13] and T at the start (other record fields fixed)
    p[P]      log multipliers of the network's P rate coefficients
    q[n, 15]  per cell xn[0..13] and T at the end

``DiffMap`` runs the forward pass (recording the ROS2S controller's accepted step
sizes) and the discrete adjoint of the recorded steps on the GPU.
``CollapseChemistry`` wraps both as a ``torch.autograd.Function``; PyTorch only
holds the device buffers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import COLLAPSE_STATE, MATH_PORTABLE, MAX_COLLAPSE_STEPS, SUCCESS, Context, WarpReactorError, lib

_declared = False


def _lib():
    global _declared
    L = lib()
    if not _declared:
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        L.wr_diff_num_multipliers.restype = i32
        L.wr_diff_create.argtypes = [i32, i32, i32, i32]
        L.wr_diff_create.restype = vp
        L.wr_diff_destroy.argtypes = [vp]
        L.wr_diff_destroy.restype = None
        L.wr_diff_last_error.argtypes = [vp]
        L.wr_diff_last_error.restype = ctypes.c_char_p
        L.wr_diff_forward.argtypes = [vp, vp, vp, vp, vp, i32, i32, vp]
        L.wr_diff_backward.argtypes = [vp, vp, vp, vp]
        L.wr_diff_record.argtypes = [vp, vp, vp]
        _declared = True
    return L


def num_multipliers() -> int:
    return _lib().wr_diff_num_multipliers()


def schedule(cells: np.ndarray, perturb: bool = True, device: int = 0) -> np.ndarray:
    """Outer schedule of a plain gridwide run of ``cells``: the grid timestep of
    every outer step (wr_grid_dt_history), trimmed to the steps taken.  The run
    uses the portable math, the arithmetic of the differentiation map."""
    with Context(len(cells), device=device, math=MATH_PORTABLE) as ctx:
        ctx.upload(np.ascontiguousarray(cells))
        rc, _ = ctx.run(perturb)
        if rc != SUCCESS:
            raise WarpReactorError(rc, "plain run for the schedule failed")
        hist = ctx.dt_history(0)
    n = int(np.argmax(hist <= 0.0)) if (hist <= 0.0).any() else MAX_COLLAPSE_STEPS
    return hist[:n].copy()


class DiffMap:
    """GPU forward map and adjoint for ``num_cells`` cells (see module docstring).

    All tensors passed in are device pointers (``int``) or objects with a
    ``data_ptr()``; ``dt_hist`` is a host float64 array."""

    def __init__(self, num_cells: int, max_outer_steps: int = MAX_COLLAPSE_STEPS,
                 max_accepted_per_cell: int = 32768, device: int = 0):
        self.n = int(num_cells)
        self.cap = int(max_accepted_per_cell)
        self.handle = _lib().wr_diff_create(self.n, int(max_outer_steps), self.cap, int(device))
        if not self.handle:
            raise WarpReactorError(-1, "wr_diff_create failed")
        self.num_multipliers = num_multipliers()
        self.nsteps = 0

    def close(self):
        if self.handle:
            _lib().wr_diff_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _err(self):
        return _lib().wr_diff_last_error(self.handle).decode()

    @staticmethod
    def _ptr(x):
        if x is None:
            return None
        return x if isinstance(x, int) else x.data_ptr()

    def forward(self, cells, u, log_mult, dt_hist, perturb, q):
        dt = np.ascontiguousarray(dt_hist, np.float64)
        rc = _lib().wr_diff_forward(self.handle, self._ptr(cells), self._ptr(u), self._ptr(log_mult),
                                    dt.ctypes.data, len(dt), int(bool(perturb)), self._ptr(q))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_diff_forward ({self._err()})")
        self.nsteps = len(dt)

    def backward(self, qbar, ubar, pbar):
        rc = _lib().wr_diff_backward(self.handle, self._ptr(qbar), self._ptr(ubar), self._ptr(pbar))
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_diff_backward ({self._err()})")

    def record(self):
        """(step sizes n x cap, counts n x nsteps) of the last forward pass."""
        hbuf = np.zeros((self.n, self.cap))
        counts = np.zeros((self.n, self.nsteps), np.int32)
        rc = _lib().wr_diff_record(self.handle, hbuf.ctypes.data, counts.ctypes.data)
        if rc != SUCCESS:
            raise WarpReactorError(rc, f"wr_diff_record ({self._err()})")
        return hbuf, counts


def initial_u(cells: np.ndarray) -> np.ndarray:
    """The map's inputs of host records: xn[0..13] and T per cell."""
    assert cells.dtype == COLLAPSE_STATE
    return np.concatenate([cells["xn"], cells["T"][:, None]], axis=1)


def _torch_function():
    import torch

    class CollapseChemistry(torch.autograd.Function):
        """q = F(u, p) on the GPU; backward runs the discrete adjoint.

        forward(u, log_mult, dmap, cells_dev, dt_hist, perturb): u (n, 15) and
        log_mult (P,) float64 CUDA tensors; cells_dev a uint8 CUDA tensor holding
        the n records (their fields other than xn and T); dt_hist a host array."""

        @staticmethod
        def forward(ctx, u, log_mult, dmap, cells_dev, dt_hist, perturb=True):
            u = u.contiguous()
            log_mult = log_mult.contiguous()
            q = torch.empty_like(u)
            torch.cuda.current_stream().synchronize()
            dmap.forward(cells_dev, u, log_mult, dt_hist, perturb, q)
            ctx.dmap = dmap
            return q

        @staticmethod
        def backward(ctx, qbar):
            dmap = ctx.dmap
            qbar = qbar.contiguous()
            ubar = torch.empty_like(qbar)
            pbar = torch.empty(dmap.num_multipliers, dtype=qbar.dtype, device=qbar.device)
            torch.cuda.current_stream().synchronize()
            dmap.backward(qbar, ubar, pbar)
            return ubar, pbar, None, None, None, None

    return CollapseChemistry


_fn = None


def collapse_chemistry(u, log_mult, dmap: DiffMap, cells_dev, dt_hist, perturb: bool = True):
    """``CollapseChemistry.apply``: differentiable final xn/T of the grid."""
    global _fn
    if _fn is None:
        _fn = _torch_function()
    return _fn.apply(u, log_mult, dmap, cells_dev, dt_hist, perturb)
