"""Differentiation form: the derivative code, the CPU map and tangent-linear, and
the GPU forward map and discrete adjoint.

The map (wr_diff.cuh): a grid advanced by the gridwide-independent kernels
(reproducer.cpp:7696-7785) through a fixed outer schedule, with log multipliers on
the network's rate coefficients and the ROS2S controller's accepted steps held
fixed.  Checks:
  * generated VJP/JVP code against finite differences and against each other;
  * the map at p = 0 reproduces the plain integrator bit for bit (CPU and GPU);
  * GPU forward == CPU map bit for bit at p != 0, same accepted steps;
  * GPU adjoint == CPU tangent-linear (inner products <qbar, dq>), and both against
    central finite differences on the smooth components (major species, T).
Trace species far below the integrator's absolute tolerance (the D-bearing
species at the reference's initial 1e-40) pass through floor kinks of the frozen
map, so finite differences of them carry no derivative information; the checks
use e-, H, H2 and T.
"""
import os

import numpy as np
import pytest

SMOOTH = [0, 2, 8, 14]  # e-, H, H2, T


@pytest.fixture(scope="module")
def diff_oracle(built):
    from oracle import oracle as O
    return O.load_diff()


@pytest.fixture(scope="module")
def grid2(oracle_port):
    from oracle import oracle as O
    cells = oracle_port.make_grid(2)
    plain = cells.copy()
    rc, hist = O.grid_schedule(oracle_port, plain)
    assert rc == 1
    return cells, plain, hist


def _states():
    """Network fixture states in the network's range (T >= 100 K), except those
    sitting exactly on a rate fit's branch temperature (100 K, 10^4 K), where
    central differences straddle the kink."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "network_ref.npz"))
    out = []
    for X, T in zip(z["X"], z["T"]):
        if np.all(X > 0) and np.isfinite(T) and T >= 100.0 and T not in (100.0, 10000.0):
            out.append((X.copy(), float(T)))
    return out[:12]


def test_multiplier_count(diff_oracle):
    assert diff_oracle.num_multipliers == 44


def test_derivative_code_against_finite_differences(diff_oracle):
    """JVPs of the RHS (with multipliers) and of the analytic Jacobian against
    central differences; VJPs against the JVPs (<fbar, J v> == <J^T fbar, v>)."""
    D = diff_oracle
    P = D.num_multipliers
    rng = np.random.default_rng(5)
    for X, T in _states():
        m = np.exp(rng.normal(0, 0.1, P))
        dX = rng.normal(size=14) * X * 1e-6
        dT = rng.normal() * T * 1e-6
        dm = rng.normal(size=P) * m * 1e-6
        fd = (D.rhs(X + dX, T + dT, m + dm) - D.rhs(X - dX, T - dT, m - dm)) / 2
        f, df = D.rhs_jvp(X, T, m, dX, dT, dm)
        assert np.array_equal(f, D.rhs(X, T, m))
        assert np.abs(df - fd).max() <= 1e-6 * np.abs(df).max()
        fb = rng.normal(size=15)
        Xb, Tb, mb = D.rhs_vjp(X, T, m, fb)
        lhs, rhs = fb @ df, Xb @ dX + Tb * dT + mb @ dm
        assert abs(lhs - rhs) <= 1e-12 * (abs(fb) @ abs(df))
        J, dJ = D.jac_jvp(X, T, dX, dT)
        Jp, _ = D.jac_jvp(X + dX, T + dT, dX, dT)
        Jm, _ = D.jac_jvp(X - dX, T - dT, dX, dT)
        assert np.abs(dJ - (Jp - Jm) / 2).max() <= 1e-6 * np.abs(dJ).max()
        Jb = rng.normal(size=(15, 15))
        Xb, Tb = D.jac_vjp(X, T, Jb)
        lhs, rhs = (Jb * dJ).sum(), Xb @ dX + Tb * dT
        assert abs(lhs - rhs) <= 1e-11 * (abs(Jb) * abs(dJ)).sum()


def test_unit_multipliers_are_the_plain_rhs(diff_oracle, oracle_port):
    for X, T in _states():
        f = diff_oracle.rhs(X, T, np.ones(diff_oracle.num_multipliers))
        assert f.tobytes() == oracle_port.net_rhs(X, T).tobytes()


def test_cpu_map_reproduces_plain_run(diff_oracle, grid2):
    cells, plain, hist = grid2
    rc, q, hbuf, counts = diff_oracle.record(cells, hist, cap=20000)
    assert rc == 1
    qp = np.concatenate([plain["xn"], plain["T"][:, None]], 1)
    assert q.tobytes() == qp.tobytes()
    assert (counts.sum(1) == plain["stats"]["accepted_steps"]).all()
    rc, q2 = diff_oracle.replay(cells, hist, hbuf, counts)
    assert rc == 1 and q2.tobytes() == q.tobytes()


def test_cpu_tangent_against_finite_differences(diff_oracle, grid2):
    """Tangent-linear of the frozen map vs central differences, 100 outer steps,
    multiplier and temperature directions, smooth components."""
    cells, _, hist = grid2
    h = hist[:100]
    rng = np.random.default_rng(11)
    lm = rng.normal(0, 0.1, diff_oracle.num_multipliers)
    rc, q, hbuf, counts = diff_oracle.record(cells, h, log_mult=lm, cap=20000)
    assert rc == 1
    u = np.concatenate([cells["xn"], cells["T"][:, None]], 1)
    dp = rng.normal(size=diff_oracle.num_multipliers)
    _, _, dq = diff_oracle.tangent(cells, h, hbuf, counts, dlog_mult=dp, log_mult=lm)
    eps = 1e-5
    _, qa = diff_oracle.replay(cells, h, hbuf, counts, log_mult=lm + eps * dp)
    _, qb = diff_oracle.replay(cells, h, hbuf, counts, log_mult=lm - eps * dp)
    fd = (qa - qb) / (2 * eps)
    assert np.abs(fd[:, SMOOTH] - dq[:, SMOOTH]).max() <= 1e-6 * np.abs(dq[:, SMOOTH]).max()
    du = np.zeros_like(u)
    du[:, 14] = u[:, 14]
    _, _, dq = diff_oracle.tangent(cells, h, hbuf, counts, du=du, log_mult=lm)
    eps = 1e-4
    _, qa = diff_oracle.replay(cells, h, hbuf, counts, u=u + eps * du, log_mult=lm)
    _, qb = diff_oracle.replay(cells, h, hbuf, counts, u=u - eps * du, log_mult=lm)
    fd = (qa - qb) / (2 * eps)
    assert np.abs(fd[:, SMOOTH] - dq[:, SMOOTH]).max() <= 1e-4 * np.abs(dq[:, SMOOTH]).max()


# ----------------------------------------------------------------------------- GPU
def _device_setup(wr, cells, torch):
    cells_dev = torch.from_numpy(np.ascontiguousarray(cells).view(np.uint8)).cuda()
    return cells_dev


@pytest.mark.gpu
def test_gpu_forward_bitwise(wr, gpu, diff_oracle, grid2):
    """GPU map == plain GPU run at p = 0; == CPU map at random p; same steps."""
    torch = pytest.importorskip("torch")
    from warp_reactor_gb300 import diff
    cells, plain, hist = grid2
    sched = diff.schedule(cells)
    assert sched.tobytes() == hist.tobytes()
    n = len(cells)
    cells_dev = _device_setup(wr, cells, torch)
    q = torch.empty((n, 15), dtype=torch.float64, device="cuda")
    with diff.DiffMap(n) as dm:
        dm.forward(cells_dev, None, None, hist, True, q)
        qp = np.concatenate([plain["xn"], plain["T"][:, None]], 1)
        assert q.cpu().numpy().tobytes() == qp.tobytes()
        # random multipliers over the first 300 outer steps (with this grid's
        # schedule, the thermally unstable cell 1 ends in the reference
        # controller's DT_UNDERFLOW near step 690 for such draws, on the CPU too)
        h = hist[:300]
        lm = np.random.default_rng(3).normal(0, 0.1, dm.num_multipliers)
        lm_dev = torch.from_numpy(lm).cuda()
        dm.forward(cells_dev, None, lm_dev, h, True, q)
        hbuf, counts = dm.record()
    rc, qo, hbo, co = diff_oracle.record(cells, h, log_mult=lm, cap=hbuf.shape[1])
    assert rc == 1
    assert (counts == co).all()
    for i, used in enumerate(counts.sum(1)):  # rows hold the last forward's steps first
        assert hbuf[i, :used].tobytes() == hbo[i, :used].tobytes()
    assert q.cpu().numpy().tobytes() == qo.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("nsteps", [100, 1000])
def test_gpu_adjoint_against_tangent_linear(wr, gpu, diff_oracle, grid2, nsteps):
    """<qbar, dq> from the CPU tangent-linear == <ubar, du> + <pbar, dp> from the
    GPU adjoint, for random directions (both differentiate the same frozen map)."""
    torch = pytest.importorskip("torch")
    from warp_reactor_gb300 import diff
    cells, _, hist = grid2
    h = hist[:nsteps]
    n = len(cells)
    rng = np.random.default_rng(nsteps)
    # the whole schedule at p = 0 (see test_gpu_forward_bitwise), 100 steps at random p
    lm = rng.normal(0, 0.1, diff_oracle.num_multipliers) if nsteps <= 100 else np.zeros(diff_oracle.num_multipliers)
    u = diff.initial_u(cells)
    cells_dev = _device_setup(wr, cells, torch)
    q = torch.empty((n, 15), dtype=torch.float64, device="cuda")
    with diff.DiffMap(n) as dm:
        dm.forward(cells_dev, torch.from_numpy(u).cuda(), torch.from_numpy(lm).cuda(), h, True, q)
        hbuf, counts = dm.record()
        qbar = np.zeros((n, 15))
        qbar[:, SMOOTH] = rng.normal(size=(n, len(SMOOTH))) / np.abs(q.cpu().numpy()[:, SMOOTH])
        # cells with several times the median work are the thermally unstable ones:
        # over the whole collapse their derivatives are conditioned beyond what two
        # FP64 evaluation orders (tangent, adjoint) agree on, so only the others
        # are seeded
        acc = counts.sum(1)
        qbar[acc > 1.5 * np.median(acc)] = 0.0
        ubar = torch.empty((n, 15), dtype=torch.float64, device="cuda")
        pbar = torch.empty(dm.num_multipliers, dtype=torch.float64, device="cuda")
        dm.backward(torch.from_numpy(qbar).cuda(), ubar, pbar)
        ubar, pbar = ubar.cpu().numpy(), pbar.cpu().numpy()
    assert np.isfinite(ubar).all() and np.isfinite(pbar).all()
    for trial in range(3):
        du = np.zeros_like(u)
        du[:, 14] = rng.normal(size=n) * u[:, 14]
        du[:, [0, 2, 8]] = rng.normal(size=(n, 3)) * u[:, [0, 2, 8]] * 1e-3
        dp = rng.normal(size=diff_oracle.num_multipliers)
        _, _, dq = diff_oracle.tangent(cells, h, hbuf, counts, du=du, dlog_mult=dp, u=u, log_mult=lm)
        tl = (qbar * dq).sum()
        adj = (ubar * du).sum() + pbar @ dp
        scale = np.abs(qbar * dq).sum()
        assert abs(tl - adj) <= 1e-8 * scale, (tl, adj, scale)


@pytest.mark.gpu
def test_torch_function_gradients(wr, gpu, diff_oracle, grid2):
    """torch.autograd through CollapseChemistry: the gradient of a log-space loss
    in the multipliers matches central differences of the same loss evaluated by
    the CPU map on the GPU-recorded steps."""
    torch = pytest.importorskip("torch")
    from warp_reactor_gb300 import diff
    cells, _, hist = grid2
    h = hist[:100]
    n = len(cells)
    cells_dev = _device_setup(wr, cells, torch)
    u_np = diff.initial_u(cells)
    rng = np.random.default_rng(9)
    lm_np = rng.normal(0, 0.1, diff_oracle.num_multipliers)
    target = np.abs(u_np[:, SMOOTH]) * 1.1
    with diff.DiffMap(n) as dm:
        lm = torch.from_numpy(lm_np).cuda().requires_grad_(True)
        u = torch.from_numpy(u_np).cuda().requires_grad_(True)
        q = diff.collapse_chemistry(u, lm, dm, cells_dev, h)
        loss = ((torch.log(q[:, SMOOTH]) - torch.log(torch.from_numpy(target).cuda())) ** 2).sum()
        loss.backward()
        g = lm.grad.cpu().numpy()
        hbuf, counts = dm.record()
    assert u.grad is not None and torch.isfinite(u.grad).all()

    def loss_cpu(p):
        rc, qq = diff_oracle.replay(cells, h, hbuf, counts, log_mult=p)
        assert rc == 1
        return ((np.log(qq[:, SMOOTH]) - np.log(target)) ** 2).sum()

    assert abs(loss_cpu(lm_np) - loss.item()) <= 1e-12 * abs(loss.item())
    d = rng.normal(size=len(lm_np))
    eps = 1e-5
    fd = (loss_cpu(lm_np + eps * d) - loss_cpu(lm_np - eps * d)) / (2 * eps)
    assert abs(fd - g @ d) <= 1e-5 * abs(fd)
