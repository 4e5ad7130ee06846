"""The spec workloads of the differentiation and batching forms on the GPU,
checked against the oracle (bench.py times the same workloads; the checks live
here so that the benchmark only measures).

* Differentiation form, 16^3 reference cells, 1,000 outer steps, 44 log
  multipliers ~ N(0, 0.1^2): on a sample of cells, the GPU adjoint against the
  CPU FP64 tangent-linear of the same frozen map (the exact check), and against
  central differences of the multiplier gradient at h = 1e-4.  Over this
  stiff 1,000-step integration the differences are rounding-limited below that:
  on this sample their error grows as 1/h (8e-7 at h = 1e-4, 4e-6 at 1e-5, 2e-5
  at 1e-6), while the adjoint stays within 1e-12 of the tangent-linear.
* Batching form at a quarter of its dimensions (32^3 + 8^3, 12^3, 20^3, 24^3
  sub-grids of the seeded log-normal density / log-uniform T workload) in one
  context: sampled cells of every grid replayed bit for bit by the oracle
  through that grid's dt history.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_differentiation_workload_gradients(wr, gpu):
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    from warp_reactor_gb300 import diff
    D = O.load_diff()
    cells = wr.make_grid(16)
    n = len(cells)
    sched = diff.schedule(cells)
    rng = np.random.default_rng(2024)
    P = diff.num_multipliers()
    lm = rng.normal(0.0, 0.1, P)
    u = diff.initial_u(cells)
    cells_dev = torch.from_numpy(np.ascontiguousarray(cells).view(np.uint8)).cuda()
    q = torch.empty((n, 15), dtype=torch.float64, device="cuda")
    smooth = [8, 0, 14]  # H2, e-, T
    with diff.DiffMap(n) as dm:
        dm.forward(cells_dev, torch.from_numpy(u).cuda(), torch.from_numpy(lm).cuda(), sched, True, q)
        hbuf, counts = dm.record()
        qn = q.cpu().numpy()
        acc = counts.sum(1)
        light = np.flatnonzero(acc <= 1.5 * np.median(acc))
        sample = np.unique(np.concatenate([[light[0], light[-1]], rng.choice(light, 14, replace=False)]))
        qbar = np.zeros((n, 15))
        qbar[sample[:, None], smooth] = rng.normal(size=(len(sample), len(smooth))) / qn[sample[:, None], smooth]
        ubar = torch.empty((n, 15), dtype=torch.float64, device="cuda")
        pbar = torch.empty(P, dtype=torch.float64, device="cuda")
        dm.backward(torch.from_numpy(qbar).cuda(), ubar, pbar)
        ubar, pbar = ubar.cpu().numpy(), pbar.cpu().numpy()
    sub = np.ascontiguousarray(cells[sample])
    ids = sample.astype(np.int32)
    u_s = u[sample]
    hb, cn = hbuf[sample], counts[sample]
    qb = qbar[sample]
    for trial in range(2):
        du = np.zeros_like(u_s)
        du[:, 14] = rng.normal(size=len(sample)) * u_s[:, 14]
        dp = rng.normal(size=P)
        rc, qs, dq = D.tangent(sub, sched, hb, cn, du=du, dlog_mult=dp, u=u_s, log_mult=lm, cell_ids=ids)
        assert rc == 1 and qs.tobytes() == qn[sample].tobytes()
        tl = (qb * dq).sum()
        adj = (ubar[sample] * du).sum() + pbar @ dp
        assert abs(tl - adj) <= 1e-8 * np.abs(qb * dq).sum(), (tl, adj)
        eps = 1e-4
        _, qa = D.replay(sub, sched, hb, cn, u=u_s, log_mult=lm + eps * dp, cell_ids=ids)
        _, qm = D.replay(sub, sched, hb, cn, u=u_s, log_mult=lm - eps * dp, cell_ids=ids)
        terms = (qb * (qa - qm)).sum(1) / (2 * eps)
        fd = terms.sum()
        assert abs(fd - pbar @ dp) <= 1e-5 * np.abs(terms).sum(), (fd, pbar @ dp)


def test_batching_workload_replay(wr, gpu, oracle_port):
    dims = [32, 8, 12, 20, 24]
    sizes = [d ** 3 for d in dims]
    parts = [wr.make_batch_grid(g, n) for g, n in enumerate(sizes)]
    cells = np.concatenate(parts)
    with wr.Context(grids=sizes, math=wr.MATH_PORTABLE) as ctx:
        ctx.upload(cells)
        best = ctx.autotune(True, steps=3)
        assert best in (0, 1, 2, 4, 5, 6, 7)  # an exact shape, never the precision form
        rc, _ = ctx.run(True)
        results = [ctx.grid_result(g) for g in range(len(sizes))]
        hists = [ctx.dt_history(g) for g in range(len(sizes))]
        ctx.download(cells)
    assert rc == wr.SUCCESS
    lib = oracle_port.lib
    lib.wro_replay.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                               ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(7)
    off = 0
    for g, n in enumerate(sizes):
        assert results[g][0] == wr.SUCCESS
        ids = np.unique(np.concatenate([[0, n - 1], rng.choice(n, min(n, 24), replace=False)])).astype(np.int32)
        sample = np.ascontiguousarray(parts[g][ids])
        r = lib.wro_replay(sample.ctypes.data, ids.ctypes.data, len(ids), 1, hists[g].ctypes.data, results[g][1],
                           os.cpu_count())
        assert r == 1
        assert sample.tobytes() == cells[off + ids].tobytes(), f"grid {g}"
        off += n
