"""The CPU oracle (test infrastructure) against the reference's own outputs.

The C-library build of the oracle must equal the reference bit for bit (golden
fixtures written by tests/golden/make_golden.py from the reference compiled from
its sources).  The portable-math build differs from it only through exp/log/cbrt.
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def grids():
    return np.load(os.path.join(GOLDEN, "grids_ref.npz"))


def test_network_bitwise(oracle_libm):
    g = np.load(os.path.join(GOLDEN, "network_ref.npz"))
    for i in range(len(g["T"])):
        J, f = oracle_libm.net_jac(g["X"][i], g["T"][i])
        assert J.tobytes() == g["J"][i].tobytes(), i
        assert f.tobytes() == g["f"][i].tobytes(), i
        assert oracle_libm.net_rhs(g["X"][i], g["T"][i]).tobytes() == g["f"][i].tobytes(), i


def test_lu_fixtures(oracle_libm, oracle_port):
    g = np.load(os.path.join(GOLDEN, "lu_ref.npz"))
    for case in range(8):
        for orc in (oracle_libm, oracle_port):
            info, LU, ip = orc.lu(g["A"][case])
            assert info == g["info"][case]
            assert LU.tobytes() == g["LU"][case].tobytes()
            assert (ip == g["ipvt"][case]).all()
            if info == 0:
                x = orc.lu_solve(LU, ip, g["b"][case])
                assert x.tobytes() == g["x"][case].tobytes()
                # residual bound of the reference's LU test (test_warp_lu.mojo:126-151)
                A, b = g["A"][case], g["b"][case]
                res = np.abs(A @ x - b).max()
                scale = max(1.0, np.abs(A).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())
                assert res <= 1e-11 * scale
    assert g["info"][1] == 15  # exactly singular last row
    assert g["ipvt"][2][0] == 1  # forced row swap


@pytest.mark.parametrize("key", ["grid1_p", "grid2_p", "grid3_p", "grid4_p", "grid2_np"])
def test_gridwide_runs_bitwise(oracle_libm, grids, key):
    ref_cells = grids[key + "_cells"]
    grid = int(key[4])
    perturb = key.endswith("_p")
    cells = oracle_libm.make_grid(grid)
    rc, cgs = oracle_libm.run(cells, perturb=perturb)
    assert rc == 1
    assert cgs == int(grids[key + "_cgs"])
    assert cells.tobytes() == ref_cells.tobytes()


def test_grid1_known_answer(oracle_libm):
    """The reference program's --grid 1 printout (438 steps, T = 3050.9215507836907)."""
    txt = open(os.path.join(GOLDEN, "grid1_stdout_ref.txt")).read().splitlines()
    vals = dict(ln.split(": ", 1) for ln in txt if ": " in ln)
    cells = oracle_libm.make_grid(1)
    rc, cgs = oracle_libm.run(cells, perturb=True)
    c = cells[0]
    assert rc == 1 and cgs == int(vals["completed global collapse steps"]) == 438
    assert repr(float(c["T"])) == vals["T"]
    assert repr(float(c["rho"])) == vals["rho"]
    assert c["stats"]["internal_steps"] == int(vals["ROS2S internal steps"])
    assert c["stats"]["jacobian_calls"] == int(vals["ROS2S jacobian calls"])
    acc, rej = vals["ROS2S accepted/rejected"].split("/")
    assert c["stats"]["accepted_steps"] == int(acc) and c["stats"]["rejected_steps"] == int(rej)


def test_portable_oracle_close_to_reference(oracle_port, grids):
    """exp/log/cbrt are the only difference from the reference CPU build: most cells
    agree to ~1e-12; an adaptive controller can amplify an ulp somewhere."""
    ref_cells = grids["grid4_p_cells"]
    cells = oracle_port.make_grid(4)
    rc, cgs = oracle_port.run(cells, perturb=True)
    assert rc == 1 and cgs == int(grids["grid4_p_cgs"])
    rT = np.abs(cells["T"] - ref_cells["T"]) / ref_cells["T"]
    assert np.median(rT) < 1e-10
    assert rT.max() < 1e-4
    assert (cells["completed_steps"] == ref_cells["completed_steps"]).all()


# ------------------------------------------------------------------ policy semantics
# Restated from the reference's grid-timestep tests
# (tests/integration/test_grid_timestep_reference.mojo:21-168) for the
# gridwide-independent policy.

def test_terminal_small_timestep_updates_driver_once(oracle_port):
    cells = oracle_port.make_grid(1)
    cells["xn"][0] = 0.0
    cells["xn"][0, 2] = 1.0e30
    cells["density_driver"][0] = 1.0e-10
    rc, dt = oracle_port.prepare(cells, 0, 0.0, 0, perturb=False)
    assert rc == 1 and dt == np.finfo(np.float64).max
    assert abs(cells["density_driver"][0] - 1.1e-10) < 1e-25


def test_invalid_density_fails(oracle_port):
    cells = oracle_port.make_grid(1)
    cells["xn"][0] = 0.0
    rc, dt = oracle_port.prepare(cells, 0, 0.0, 0, perturb=False)
    assert rc == -1


def test_density_limit_stops_before_burn(oracle_port):
    cells = oracle_port.make_grid(1)
    cells["density_driver"][0] = 1.99e-6
    rc, dt = oracle_port.prepare(cells, 0, 0.0, 0, perturb=False)
    assert rc == 1
    rc, n = oracle_port.advance(cells, 0, dt, dt)
    assert rc == 1 and n == 0
    assert cells["density_driver"][0] > 2.0e-6
    assert cells["completed_steps"][0] == 0


def test_no_active_cells_terminates(oracle_port):
    cells = oracle_port.make_grid(1)
    cells = np.concatenate([cells, cells])
    cells["xn"][:] = 0.0
    cells["xn"][:, 2] = 1.0e30
    cells["density_driver"][:] = 1.0e-10
    rc, cgs = oracle_port.run(cells, perturb=False)
    assert rc == 1 and cgs == 0
    assert (cells["completed_steps"] == 0).all() and (cells["time"] == 0.0).all()


def test_stable_minimum_and_denser_cells(oracle_port):
    base = oracle_port.make_grid(1)
    cells = np.repeat(base, 33)
    cells["xn"][31:33] *= 4.0
    rc, dt = oracle_port.prepare(cells.copy(), 0, 0.0, 0, perturb=False)
    one = np.repeat(base, 1)
    one["xn"][0] *= 4.0
    rc1, dt1 = oracle_port.prepare(one, 0, 0.0, 0, perturb=False)
    assert rc == rc1 == 1 and dt == dt1  # the denser cells set the grid dt


@pytest.mark.parametrize("count", [1, 7, 8, 31, 32, 33])
def test_partial_sizes_share_exact_output_time(oracle_port, count):
    cells = np.repeat(oracle_port.make_grid(1), count)
    rc, dt = oracle_port.prepare(cells, 0, 0.0, 0, perturb=False)
    rc2, n = oracle_port.advance(cells, 0, 0.0 + dt, dt)
    assert rc == rc2 == 1 and n == count
    assert (cells["time"] == dt).all() and (cells["completed_steps"] == 1).all()


@pytest.mark.parametrize("grid", [2, 3])
def test_legacy_local_matches_reference_program(oracle_libm, grid):
    """The oracle's legacy-local loop (the reference CPU program's default policy)
    writes the same final_states_grid<N>_cpu.bin as the reference program."""
    import warp_reactor_gb300 as wr
    ref = np.fromfile(os.path.join(GOLDEN, f"legacy_grid{grid}_ref.bin"), wr.PACKED_FINAL_STATE)
    cells = oracle_libm.make_grid(grid)
    rc, cgs = oracle_libm.run_legacy(cells, perturb=True)
    assert rc == 1
    assert wr.pack_final_states(cells, grid).tobytes() == ref.tobytes()


@pytest.mark.parametrize("count", [1, 31, 32, 33])
def test_cta32_tiles_share_one_controller(oracle_port, count):
    """gridwide-structured-cta32 restated (structured_cuda.cuh:393-782): the cells
    of a 32-cell tile take the same substeps (same counters, while every cell of
    the tile still participates: the first 200 outer steps), partial tiles work,
    and the result stays near the gridwide-independent one (the tile controller
    changes trajectories, not the physics)."""
    a = np.repeat(oracle_port.make_grid(1), count)
    b = a.copy()
    rc_i, cgs_i = oracle_port.run(a, perturb=True, nthreads=4, max_steps=200)
    rc_t, cgs_t = oracle_port.run_cta32(b, perturb=True, nthreads=4, max_steps=200)
    assert rc_i == rc_t == 1 and cgs_i == cgs_t
    st = b["stats"]
    for t in range(0, count, 32):
        tile = st[t:t + 32]
        for f in ("internal_steps", "accepted_steps", "rejected_steps", "jacobian_calls"):
            assert (tile[f] == tile[f][0]).all()
    assert np.abs(b["T"] / a["T"] - 1).max() < 1e-4
    assert (b["completed_steps"] == a["completed_steps"]).all()


def test_precision_oracle_bounded(oracle_prec, oracle_port):
    """The precision form's arithmetic (FP32 factorisation in error-weighted
    variables, one FP64 residual sweep) integrates the grid-1 collapse: more
    attempts than FP64 but within 3x (unweighted FP32 factors take ~50x), and a
    final T within 1e-3 of the FP64 oracle."""
    a = oracle_prec.make_grid(1)
    b = oracle_port.make_grid(1)
    rc_a, cgs_a = oracle_prec.run(a)
    rc_b, cgs_b = oracle_port.run(b)
    assert rc_a == rc_b == 1 and cgs_a == cgs_b == 438
    att_a, att_b = int(a["stats"]["internal_steps"].sum()), int(b["stats"]["internal_steps"].sum())
    assert att_b < att_a < 3 * att_b
    assert abs(a["T"][0] / b["T"][0] - 1) < 1e-3
