"""GPU parity: the CUDA library through its C ABI against the CPU oracle.

Integer/index results (steps, counters, pivots) must match exactly.  In portable math
the library's arithmetic is the oracle's, so floating-point results must match bit
for bit too; the CUDA-libm mode (the default) is compared with the reference's own
CUDA kernel outputs (fixtures from the reference run on GB300).
"""
import ctypes
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
pytestmark = pytest.mark.gpu


def _diag_network(wr, X, T, math):
    L = wr.lib()
    L.wr_diag_network.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 2 + [ctypes.c_int] + [ctypes.c_void_p] * 3
    n = len(T)
    X = np.ascontiguousarray(X, np.float64)
    T = np.ascontiguousarray(T, np.float64)
    J = np.zeros((n, 15, 15))
    f = np.zeros((n, 15))
    g = np.zeros((n, 15))
    assert L.wr_diag_network(n, X.ctypes.data, T.ctypes.data, math, J.ctypes.data, f.ctypes.data, g.ctypes.data) == 1
    return J, f, g


def _states(n, seed):
    rng = np.random.default_rng(seed)
    return 10.0 ** rng.uniform(-40, 18, size=(n, 14)), 10.0 ** rng.uniform(0.5, 5.0, size=n)


def test_network_portable_bitwise(wr, gpu, oracle_port):
    g = np.load(os.path.join(GOLDEN, "network_ref.npz"))
    Xr, Tr = _states(2000, 99)
    X = np.vstack([g["X"], Xr])
    T = np.concatenate([g["T"], Tr])
    J, f, f2 = _diag_network(wr, X, T, wr.MATH_PORTABLE)

    def same(a, b):
        # bit-identical, except that a NaN matches any NaN: x86 and the GPU write
        # different default-NaN bit patterns for invalid operations (adversarial
        # random states reach inf - inf; integration states never do)
        a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
        return bool(((a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))).all())

    assert same(f, f2)  # the fused J+RHS evaluation gives the RHS-only values
    for i in range(len(T)):
        Jo, fo = oracle_port.net_jac(X[i], T[i])
        assert same(J[i], Jo), i
        assert same(f[i], fo), i



def test_network_cuda_math_close_to_reference(wr, gpu):
    """CUDA's exp/log are not the C library's: values agree to a few ulps."""
    g = np.load(os.path.join(GOLDEN, "network_ref.npz"))
    J, f, _ = _diag_network(wr, g["X"], g["T"], wr.MATH_CUDA)
    for ours, ref in ((J.reshape(len(J), -1), g["J"].reshape(len(J), -1)), (f, g["f"])):
        big = np.abs(ref) > 1e-280
        rel = np.abs(ours[big] - ref[big]) / np.abs(ref[big])
        assert np.median(rel) < 1e-15 and rel.max() < 1e-9


def test_lu_fixtures_bitwise(wr, gpu):
    g = np.load(os.path.join(GOLDEN, "lu_ref.npz"))
    rng = np.random.default_rng(7)
    extra = rng.normal(size=(61, 15, 15)) + 3 * np.eye(15)
    A = np.ascontiguousarray(np.concatenate([g["A"], extra]))
    b = np.ascontiguousarray(np.concatenate([g["b"], rng.normal(size=(61, 15))]))
    n = len(A)
    LU = np.zeros_like(A)
    ip = np.zeros((n, 15), np.int32)
    info = np.zeros(n, np.int32)
    x = np.zeros_like(b)
    L = wr.lib()
    L.wr_diag_lu.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6
    assert L.wr_diag_lu(n, A.ctypes.data, b.ctypes.data, LU.ctypes.data, ip.ctypes.data, info.ctypes.data,
                        x.ctypes.data) == 1
    assert (info[:8] == g["info"]).all()
    assert LU[:8].tobytes() == g["LU"].tobytes()
    assert (ip[:8] == g["ipvt"]).all()
    ok = g["info"] == 0
    assert x[:8][ok].tobytes() == g["x"][ok].tobytes()
    from oracle import oracle
    o = oracle.load("port")
    for i in range(8, n):
        inf, LUo, ipo = o.lu(A[i])
        assert inf == info[i] and LUo.tobytes() == LU[i].tobytes() and (ipo == ip[i]).all()
        assert o.lu_solve(LUo, ipo, b[i]).tobytes() == x[i].tobytes()


def _y_states(n, seed):
    rng = np.random.default_rng(seed)
    X = 10.0 ** rng.uniform(-30, 2, size=(n, 14))
    e = 10.0 ** rng.uniform(9, 12, size=(n, 1))
    return np.hstack([X, e])


def _same(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return bool(((a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))).all())


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_coop_network_bitwise(wr, gpu, oracle_port, lanes):
    """The cooperative advance's vector programs on the GPU (burn_state_from_y +
    Jacobian + RHS, and burn_state_from_y + RHS) equal the oracle's jacobian(y) /
    rhs(y) bit for bit, integration states of a grid-2 run included."""
    ys = _y_states(300, 5)
    for steps in (150, 300, 450):
        cells = oracle_port.make_grid(2)
        oracle_port.run(cells, max_steps=steps)
        ys = np.vstack([ys, np.hstack([cells["xn"], cells["e"][:, None]])])
    ys = np.ascontiguousarray(ys)
    n = len(ys)
    J = np.zeros((n, 225))
    f = np.zeros((n, 15))
    f2 = np.zeros((n, 15))
    L = wr.lib()
    L.wr_diag_coop_network.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    assert L.wr_diag_coop_network(lanes, n, ys.ctypes.data, wr.MATH_PORTABLE, J.ctypes.data, f.ctypes.data,
                                  f2.ctypes.data) == 1
    for i in range(n):
        assert _same(J[i], oracle_port.jac(ys[i])), i
        fo = oracle_port.rhs(ys[i])
        assert _same(f[i], fo) and _same(f2[i], fo), i


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_coop_lu_fixtures_bitwise(wr, gpu, oracle_port, lanes):
    """The warp-cooperative LU and solves on the reference's LU fixtures
    (tests/gpu/test_warp_lu.mojo:19-47 of the reference) and 61 random systems."""
    g = np.load(os.path.join(GOLDEN, "lu_ref.npz"))
    rng = np.random.default_rng(7)
    extra = rng.normal(size=(61, 15, 15)) + 3 * np.eye(15)
    A = np.ascontiguousarray(np.concatenate([g["A"], extra]))
    b = np.ascontiguousarray(np.concatenate([g["b"], rng.normal(size=(61, 15))]))
    n = len(A)
    LU = np.zeros_like(A)
    ip = np.zeros((n, 15), np.int32)
    info = np.zeros(n, np.int32)
    x = np.zeros_like(b)
    L = wr.lib()
    L.wr_diag_coop_lu.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6
    assert L.wr_diag_coop_lu(lanes, n, A.ctypes.data, b.ctypes.data, LU.ctypes.data, ip.ctypes.data,
                             info.ctypes.data, x.ctypes.data) == 1
    assert (info[:8] == g["info"]).all()
    assert LU[:8].tobytes() == g["LU"].tobytes()
    assert (ip[:8] == g["ipvt"]).all()
    ok = g["info"] == 0
    assert x[:8][ok].tobytes() == g["x"][ok].tobytes()
    for i in range(8, n):
        inf, LUo, ipo = oracle_port.lu(A[i])
        assert inf == info[i] and LUo.tobytes() == LU[i].tobytes() and (ipo == ip[i]).all()
        assert oracle_port.lu_solve(LUo, ipo, b[i]).tobytes() == x[i].tobytes()


@pytest.mark.parametrize("grid,perturb", [(1, True), (2, True), (3, True), (4, True), (5, True), (2, False),
                                          (8, True)])
def test_grid_runs_bitwise(wr, gpu, oracle_port, grid, perturb):
    cells = wr.make_grid(grid)
    rc, cgs = wr.run_cells(cells, perturb, math=wr.MATH_PORTABLE)
    ref = oracle_port.make_grid(grid)
    rc_o, cgs_o = oracle_port.run(ref, perturb=perturb)
    assert rc == rc_o == wr.SUCCESS
    assert cgs == cgs_o
    assert (cells["completed_steps"] == ref["completed_steps"]).all()
    assert (cells["stats"] == ref["stats"]).all()  # substep counts
    assert cells.tobytes() == ref.tobytes()


def test_host_stepped_api_equals_device_loop(wr, gpu):
    """wr_prepare / wr_advance driven from the host like run_cells_cuda's loop
    (reproducer.cpp:7859-7959) gives the same states as the device-driven wr_run."""
    grid = 3
    a = wr.make_grid(grid)
    rc, cgs = wr.run_cells(a, True)
    b = wr.make_grid(grid)
    with wr.Context(len(b)) as ctx:
        ctx.upload(b)
        grid_time, done = 0.0, 0
        for step in range(wr.MAX_COLLAPSE_STEPS):
            r, dt = ctx.prepare(done, grid_time, step, True)
            assert r == wr.SUCCESS
            if dt == np.finfo(np.float64).max:
                break
            r, n = ctx.advance(done, grid_time + dt, dt)
            assert r == wr.SUCCESS
            if n == 0:
                break
            grid_time += dt
            done += 1
        ctx.download(b)
    assert done == cgs
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("grid,variant", [(4, None), (8, None), (4, 2), (4, 5), (4, 7)])
def test_cuda_math_equals_reference_cuda_kernel(wr, gpu, grid, variant):
    """WR_MATH_CUDA reproduces the reference's own CUDA kernels (reproducer.cpp
    compiled with nvcc --fmad=false for sm_103a and run on GB300) bit for bit:
    the default (cooperative, 16 lanes per cell) advance, the lane-per-cell
    advance (variant 2) and the cooperative advance with 8 and 32 lanes."""
    path = os.path.join(GOLDEN, f"refcuda_grid{grid}.bin")
    ref = np.fromfile(path, wr.PACKED_FINAL_STATE)
    cells = wr.make_grid(grid)
    with wr.Context(len(cells), 0, wr.MATH_CUDA) as ctx:
        if variant is not None:
            ctx.set_variant(variant)
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        ctx.download(cells)
    assert rc == wr.SUCCESS
    assert wr.pack_final_states(cells, grid).tobytes() == ref.tobytes()


def test_failure_bad_inputs_is_reported(wr, gpu):
    """A host-made invalid cell (zero density, reproducer.cpp:7721-7725) ends the
    run with BAD_INPUTS, like the reference; the context stays usable."""
    cells = wr.make_grid(2)
    cells["xn"][5] = 0.0
    with wr.Context(len(cells)) as ctx:
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        assert rc == wr.BAD_INPUTS and cgs == 0
        good = wr.make_grid(2)
        ctx.upload(good)
        rc, cgs = ctx.run(True)
        assert rc == wr.SUCCESS and cgs == 1000


def test_failure_time_mismatch(wr, gpu):
    cells = wr.make_grid(2)
    cells["time"][3] = 1.0  # a participating cell out of step with the grid clock
    rc, cgs = wr.run_cells(cells, True)
    assert rc == wr.BAD_INPUTS and cgs == 0


def test_full_grid_64_replay_sample(wr, gpu, oracle_port):
    """64^3 (the benchmark size): the oracle replays a sample of cells through the
    GPU's grid-dt history and must reproduce them bit for bit; the sample includes
    the cells that set the grid dt."""
    grid = 64
    cells = wr.make_grid(grid)
    with wr.Context(len(cells), 0, wr.MATH_PORTABLE) as ctx:
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        hist = np.zeros(wr.MAX_COLLAPSE_STEPS)
        L = wr.lib()
        L.wr_dt_history.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        assert L.wr_dt_history(ctx.handle, hist.ctypes.data, len(hist)) == 1
        ctx.download(cells)
    assert rc == wr.SUCCESS and cgs == 1000
    rng = np.random.default_rng(64)
    ids = np.unique(np.concatenate([[0, len(cells) - 1], rng.choice(len(cells), 48, replace=False)]))
    sample = np.repeat(oracle_port.make_grid(1), len(ids))
    lib = oracle_port.lib
    lib.wro_replay.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                               ctypes.c_int, ctypes.c_int]
    ids32 = np.ascontiguousarray(ids, np.int32)
    r = lib.wro_replay(sample.ctypes.data, ids32.ctypes.data, len(ids), 1, hist.ctypes.data, cgs, os.cpu_count())
    assert r == 1
    assert sample.tobytes() == cells[ids].tobytes()
    # grid-wide invariants
    assert np.isfinite(cells["T"]).all() and (cells["xn"] > 0).all()
    live = cells["completed_steps"] == cgs
    assert (cells["time"][live] == cells["time"][live][0]).all()


@pytest.mark.parametrize("variant", [0, 1, 2, 4, 5, 7])
def test_advance_variants_identical(wr, gpu, variant):
    """Every launch shape of the advance kernel gives the same bits."""
    a = wr.make_grid(3)
    rc0, cgs0 = wr.run_cells(a, True)
    b = wr.make_grid(3)
    with wr.Context(len(b)) as ctx:
        ctx.set_variant(variant)
        ctx.upload(b)
        rc, cgs = ctx.run(True)
        ctx.download(b)
    assert rc == rc0 == wr.SUCCESS and cgs == cgs0
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("variant", [5, 6, 7])
def test_phase_counters_keep_results(wr, gpu, variant):
    """The cooperative advance with its phase counters on (the instrumented
    instantiation, inside the captured graph of wr_run) gives the same bits as
    without; the counters cover every phase and count the attempts."""
    a = wr.make_grid(3)
    rc0, cgs0 = wr.run_cells(a, True)
    b = wr.make_grid(3)
    with wr.Context(len(b)) as ctx:
        ctx.set_variant(variant)
        ctx.phase_counters(True)
        ctx.upload(b)
        rc, cgs = ctx.run(True)
        ph = ctx.read_phases(reset=True)
        again = ctx.read_phases()
        ctx.download(b)
        ctx.phase_counters(False)
    assert rc == rc0 == wr.SUCCESS and cgs == cgs0
    assert a.tobytes() == b.tobytes()
    phases = [ph[k] for k in wr.Context.PHASES]
    assert all(v > 0 for v in phases[1:]), ph
    assert sum(phases) <= ph["cycles"]
    assert 0 < ph["attempts"] <= int(b["stats"]["internal_steps"].sum())
    assert ph["warps"] > 0 and all(v == 0 for v in again.values())


def test_precision_form_against_its_oracle(wr, gpu, oracle_prec, oracle_port):
    """The precision form (advance variant 3: FP32 factorisation in error-weighted
    variables + one FP64 residual sweep per stage solve) equals its own oracle
    restatement bit for bit over 40 outer steps of a 2^3 grid, substep counts
    included; against the FP64 oracle its final state stays within 1e-2 (the
    form's error over a whole collapse is measured by bench.py)."""
    cells = wr.make_grid(2)
    ref = oracle_prec.make_grid(2)
    fp64 = oracle_port.make_grid(2)
    gt, gt_o, cgs = 0.0, 0.0, 0
    with wr.Context(len(cells), 0, wr.MATH_PORTABLE) as ctx:
        ctx.set_variant(3)
        ctx.upload(cells)
        for step in range(40):
            rc, dt = ctx.prepare(cgs, gt, step, True)
            rc_o, dt_o = oracle_prec.prepare(ref, cgs, gt_o, step, True)
            assert rc == rc_o == wr.SUCCESS and dt == dt_o
            rc, cnt = ctx.advance(cgs, gt + dt, dt)
            rc_o, cnt_o = oracle_prec.advance(ref, cgs, gt_o + dt_o, dt_o)
            assert rc == rc_o == wr.SUCCESS and cnt == cnt_o
            gt += dt
            gt_o += dt_o
            cgs += 1
        ctx.download(cells)
    assert cells.tobytes() == ref.tobytes()
    oracle_port.run(fp64, max_steps=40)
    rT = np.abs(cells["T"] - fp64["T"]) / fp64["T"]
    big = fp64["xn"] > 1e-20
    rx = np.abs(cells["xn"] - fp64["xn"])[big] / fp64["xn"][big]
    assert rT.max() < 1e-2 and np.median(rx) < 1e-2


def test_batched_grids_equal_separate_runs(wr, gpu, oracle_port):
    """Batching form: grids of 2^3, 3^3 and 4^3 cells in one context (one launch per
    kernel for all of them) give, grid by grid, the bits of separate runs; a grid
    with the batching workload's seeded log-normal density / log-uniform T is
    checked against the oracle."""
    sizes = [8, 27, 64, 125]
    parts = [wr.make_grid(2), wr.make_grid(3), wr.make_grid(4), wr.make_batch_grid(3, 125)]
    cells = np.concatenate(parts)
    with wr.Context(grids=sizes, math=wr.MATH_PORTABLE) as ctx:
        ctx.upload(cells)
        rc, _ = ctx.run(True)
        results = [ctx.grid_result(g) for g in range(len(sizes))]
        ctx.download(cells)
    assert rc == wr.SUCCESS
    off = 0
    for g, part in enumerate(parts):
        ref = part.copy()
        rc_o, cgs_o = oracle_port.run(ref, perturb=True)
        assert results[g] == (rc_o, cgs_o)
        assert cells[off:off + sizes[g]].tobytes() == ref.tobytes(), g
        off += sizes[g]


def test_autotuner_keeps_results(wr, gpu):
    """The autotuner times the launch shapes on a copy of the state and leaves the
    state untouched; the run after it gives the same bits as an untuned run."""
    a = wr.make_grid(3)
    wr.run_cells(a, True)
    b = wr.make_grid(3)
    with wr.Context(len(b)) as ctx:
        ctx.upload(b)
        best = ctx.autotune(True, steps=3)
        assert best in (0, 1, 2, 4, 5, 6, 7)
        rc, cgs = ctx.run(True)
        ctx.download(b)
    assert rc == wr.SUCCESS and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("grid", [2, 3])
def test_legacy_local_policy_bitwise(wr, gpu, oracle_port, grid):
    """WR_POLICY_LEGACY_LOCAL on the GPU equals the oracle's legacy-local loop (the
    reference CPU program's default policy) bit for bit."""
    cells = wr.make_grid(grid)
    with wr.Context(len(cells), 0, wr.MATH_PORTABLE) as ctx:
        ctx.set_policy(wr.POLICY_LEGACY_LOCAL)
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        ctx.download(cells)
    ref = oracle_port.make_grid(grid)
    rc_o, cgs_o = oracle_port.run_legacy(ref, perturb=True)
    assert rc == rc_o == wr.SUCCESS and cgs == cgs_o
    assert cells.tobytes() == ref.tobytes()


@pytest.mark.parametrize("grid", [4, 8])
def test_cta32_policy_equals_reference_structured_kernel(wr, gpu, grid):
    """WR_POLICY_GRIDWIDE_CTA32 with CUDA math reproduces the reference's own
    structured CUDA kernel (advance_collapse_gridwide_structured_kernel,
    structured_cuda.cuh:393-782, built with the slice headers of the reference's
    tools/slice_dag.py and run on GB300) bit for bit."""
    path = os.path.join(GOLDEN, f"refstructured_grid{grid}.bin")
    ref = np.fromfile(path, wr.PACKED_FINAL_STATE)
    cells = wr.make_grid(grid)
    with wr.Context(len(cells), 0, wr.MATH_CUDA) as ctx:
        ctx.set_policy(wr.POLICY_GRIDWIDE_CTA32)
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        ctx.download(cells)
    assert rc == wr.SUCCESS
    assert wr.pack_final_states(cells, grid).tobytes() == ref.tobytes()


@pytest.mark.parametrize("grid", [3, 4])  # a partial tile of 27 cells; two full tiles
def test_cta32_policy_bitwise(wr, gpu, oracle_port, grid):
    """WR_POLICY_GRIDWIDE_CTA32 (one controller per 32-cell tile, the reference's
    structured CUDA policy) on the GPU equals the oracle's restatement bit for bit;
    grid 5 ends in a partial tile (125 = 3 x 32 + 29 cells)."""
    cells = wr.make_grid(grid)
    with wr.Context(len(cells), 0, wr.MATH_PORTABLE) as ctx:
        ctx.set_policy(wr.POLICY_GRIDWIDE_CTA32)
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        ctx.download(cells)
    ref = oracle_port.make_grid(grid)
    rc_o, cgs_o = oracle_port.run_cta32(ref, perturb=True)
    assert rc == rc_o == wr.SUCCESS and cgs == cgs_o
    assert cells.tobytes() == ref.tobytes()
