"""wr_advance_cells_noalloc: the advance step for callers that cannot allocate.

Such callers keep their cells in device memory owned by someone else (another
framework's allocator or pool, a budgeted device) and may not call cudaMalloc.
The entry point takes their device records, uses only the library's fixed
file-scope scratch array, and must give exactly what the context entry point
(wr_prepare / wr_advance) gives.  This file is collected last on purpose.
"""
import ctypes
import os

import numpy as np
import pytest


def _cudart(wr):
    from warp_reactor_gb300 import build
    for path in ("libcudart.so", os.path.join(build._cuda_home(), "lib64", "libcudart.so")):
        try:
            return ctypes.CDLL(path)
        except OSError:
            continue
    pytest.fail("libcudart not found")


def _noalloc(wr):
    f = wr.lib().wr_advance_cells_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_int)]
    wr.lib().wr_noalloc_last_error.restype = ctypes.c_char_p
    return f


def test_noalloc_rejects_oversize(wr):
    f = _noalloc(wr)
    n = ctypes.c_int(0)
    rc = f(ctypes.c_void_p(16), 4097, 0, 1.0, 1.0, ctypes.byref(n))
    assert rc == wr.BAD_INPUTS
    assert b"exceeds the no-allocation limit of 4096" in wr.lib().wr_noalloc_last_error()


@pytest.mark.gpu
def test_noalloc_advance_matches_context_advance(wr, gpu):
    cudart = _cudart(wr)
    f = _noalloc(wr)
    H2D, D2H = 1, 2
    cells = wr.make_grid(8)
    nbytes = cells.nbytes
    dptr = ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(dptr), ctypes.c_size_t(nbytes)) == 0  # the caller's own buffer
    try:
        with wr.Context(len(cells), 0, wr.MATH_PORTABLE) as ctx:
            ctx.upload(cells)
            done, grid_time = 0, 0.0
            for step in range(2):  # two calls in a row
                rc, dt = ctx.prepare(done, grid_time, step, True)
                assert rc == wr.SUCCESS
                pre = np.empty_like(cells)
                ctx.download(pre)
                rc, n_ctx = ctx.advance(done, grid_time + dt, dt)
                assert rc == wr.SUCCESS and n_ctx == len(cells)
                want = np.empty_like(cells)
                ctx.download(want)

                assert cudart.cudaMemcpy(dptr, pre.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(nbytes), H2D) == 0
                n = ctypes.c_int(-1)
                rc2 = f(dptr, len(cells), done, grid_time + dt, dt, ctypes.byref(n))
                assert rc2 == wr.SUCCESS, wr.lib().wr_noalloc_last_error()
                got = np.empty_like(cells)
                assert cudart.cudaMemcpy(got.ctypes.data_as(ctypes.c_void_p), dptr, ctypes.c_size_t(nbytes), D2H) == 0
                assert n.value == n_ctx
                assert got.tobytes() == want.tobytes()  # bit for bit, like every other parity test
                last = (pre, done, grid_time + dt, dt)
                done += 1
                grid_time += dt
        # No allocation: free device memory before and after several calls in a
        # row with nothing else in between (cudaMemGetInfo is device-wide, so an
        # allocation by any other user of the GPU in between would show as well).
        free0, free1, total_b = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        assert cudart.cudaMemGetInfo(ctypes.byref(free0), ctypes.byref(total_b)) == 0
        pre, cgs, next_time, dt = last
        for _ in range(3):  # the last step again, from its own input state
            assert cudart.cudaMemcpy(dptr, pre.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(nbytes), H2D) == 0
            n = ctypes.c_int(-1)
            assert f(dptr, len(cells), cgs, next_time, dt, ctypes.byref(n)) == wr.SUCCESS
        assert cudart.cudaMemGetInfo(ctypes.byref(free1), ctypes.byref(total_b)) == 0
        assert free1.value == free0.value
    finally:
        cudart.cudaFree(dptr)
