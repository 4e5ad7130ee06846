#!/usr/bin/env python3
"""Benchmark: cells/s of the 64^3 gridwide-independent primordial-chemistry collapse.

One *step* is one full collapse of the grid: 64^3 = 262,144 cells from the
reference's initial condition through the 1,000-outer-step free-fall schedule with
seeded perturbations (the reference's config ``--grid 64``), plain FP64 with
CUDA's exp/log -- the arithmetic of the reference's own CUDA build, so the final
states equal the reference CUDA kernel's bit for bit.  The metric is the
reference's: cells / integration time (reproducer.cpp:8626-8651; published 15,055
cells/s on H200, docs/performance/optimization-results.md:51).

  value   device time of wr_run (the shipped path: CUDA-graph replay of the outer
          steps), an event pair on the library's stream around the whole run, with
          the state already in HBM; L2 is flushed (256 MiB write) before each step
  e2e     the same through the public API with host buffers: create, H2D of the
          216-byte records, run, D2H, destroy (wall clock)
  roofline  the advance kernel, FP64-bound: algorithmic FP64 work (the reference's
          source-level operation counts, weighted exp/log = 25, sqrt/cbrt = 20,
          + - * / = 1, times the per-cell Jacobian and attempt counters) over its
          duration (event nodes inside the graph around every advance launch),
          against this GPU's measured FP64 FMA rate; beside it the generated
          programs' steps, FP64 issue slots and modelled shared-memory
          wavefronts per attempt (programs_per_attempt)
  substeps  ROS2S attempts, accepted, rejected (exact: attempts - accepted) and
          Jacobians of the timed run, summed over cells
  cpu_baseline  the CPU oracle with C-library math (bitwise the reference's CPU
          arithmetic) on all host cores, on a 16^3 full collapse

``forms`` in the line, each after the timed region and within a wall-clock budget
(``--budget-s``): the reference's own CUDA kernels on the same grid and GPU (their
time, and whether the final states equal this run's byte for byte), the portable
exp/log mode with its error against the reference's result, the precision form,
the gridwide-structured-cta32 policy, the differentiation form (16^3) and the
batching form (``--forms-batch-scale``).

``--impl reference`` times the reference's CPU path (the same CPU oracle) instead:
each step is a 16^3 full collapse on all host cores.  Other modes: ``--diff``,
``--batch``, ``--probe-fp64``, the profiling drivers ``--profile-steps`` and
``--profile-policy``, and ``--profile-phases`` (the cooperative advance's phase
counters over one collapse).

Multi-GPU: the path does not shard (every outer step needs the grid-wide minimum
over all cells); N > 1 runs N independent replicas, one per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PUBLISHED_CELLS_PER_S = 15055.0  # H200, docs/performance/optimization-results.md:51 of the reference
F_JAC_EXTRA = 104   # burn_state_from_y before each Jacobian (eos_re sums), reproducer.cpp:7029-7038
F_RHS_EXTRA = 104   # the same before each RHS
F_LU = 2149         # lu_decomposition<15>: sum_{m=1..14} (1 div + m mul + 2 m^2), reproducer.cpp:96-151
F_SOLVE = 435       # lu_solve<15>: 210 forward + 15 div + 210 backward, reproducer.cpp:154-181
F_ATTEMPT = 541     # stage combinations 375, error norm 96, controller + E = -J + I/(h gamma) 70


def _dist():
    """Rank, world size, local rank and the process group of a torchrun launch
    (one replica per GPU).  NCCL on GPUs; gloo where CUDA is absent (CPU tests
    of the multi-rank path) or when WR_DIST_BACKEND says so."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as tdist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = os.environ.get("WR_DIST_BACKEND") or ("nccl" if torch.cuda.is_available() else "gloo")
    if backend == "nccl":
        torch.cuda.set_device(local)
    tdist.init_process_group(backend)
    return rank, ws, local, tdist


def _on_gpu(tdist):
    return tdist is not None and tdist.get_backend() == "nccl"


def _barrier(tdist):
    """Barrier with the device drained on both sides (the timed region's edges)."""
    if tdist is not None:
        import torch
        if _on_gpu(tdist):
            torch.cuda.synchronize()
        tdist.barrier()
        if _on_gpu(tdist):
            torch.cuda.synchronize()


def _max_over_ranks(tdist, value):
    if tdist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if _on_gpu(tdist) else "cpu")
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(tdist, world, steps, cells_per_rank, local_seconds):
    """cells/s of the whole job: every rank's cells over the slowest rank's time."""
    return world * steps * cells_per_rank / _max_over_ranks(tdist, local_seconds)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_ops(cells):
    """Weighted FP64 operations of the reference algorithm for the work the cells did."""
    from warp_reactor_gb300.gen import build_network, ir_io
    c = build_network.op_counts(ir_io.load())
    f_j = c["source_jac_weighted"] + F_JAC_EXTRA
    f_rhs = c["source_rhs_weighted"] + F_RHS_EXTRA
    f_att = 3 * f_rhs + F_LU + 3 * F_SOLVE + F_ATTEMPT
    st = cells["stats"]
    nj = float(st["jacobian_calls"].sum())
    na = float(st["internal_steps"].sum())
    # the generated (CSE'd) counts, for reference: the fraction is computed on the
    # reference's source-level work, so CSE shows as speed, not as lost work
    cse = {"F_J_plus_RHS_cse": c["cse_jac_rhs_weighted"], "F_RHS_cse": c["cse_rhs_weighted"]}
    return nj * f_j + na * f_att, {"F_J": f_j, "F_RHS": f_rhs, "F_attempt": f_att, "jacobians": nj, "attempts": na,
                                   **cse}


def program_figures(G=16):
    """Figures of the default advance's generated vector programs (16 lanes per
    cell, two cells per warp) per ROS2S attempt of one warp: steps and FP64 issue
    slots of one Jacobian+RHS and two RHS programs, the slots per cell, and the
    shared-memory wavefronts their slot accesses take per half warp against one
    per access (coop.shared_wavefronts: the bank-conflict model)."""
    from warp_reactor_gb300.gen import coop, ir_io
    g = coop.generate(G, ir_io.load())
    out = {"lanes_per_cell": G, "slots_per_cell": g["nv"], "warps_per_sm": g["warps"], "steps": 0,
           "fp64_issue_slots": 0.0, "shared_wavefronts": 0, "shared_accesses": 0}
    for kind, runs in (("jrhs", 1), ("rhs", 2)):
        pr = g["progs"][kind]
        w = coop.shared_wavefronts(pr)
        out["steps"] += runs * pr["nsteps"]  # as executed: padded to a multiple of four
        out["fp64_issue_slots"] += runs * pr["stats"]["fp64_slots"]
        out["shared_wavefronts"] += runs * w["wavefronts"]
        out["shared_accesses"] += runs * w["ideal"]
    return out


def precision_form(wr, device, math_mode, grid=16, steps=300):
    """The precision form (advance variant 3: FP32 factorisation + one FP64 residual
    refinement per stage solve) next to the plain FP64 form (the default advance) on
    the first ``steps``
    outer steps of a ``grid``^3 collapse (host-stepped wr_prepare / wr_advance, wall
    clock of synchronous calls): speed, attempts, and the final-state error of the
    precision form against the FP64 result.  A bounded case: the FP32 factorisation
    error dominates the ROS2S error estimate and multiplies the attempts, so a full
    64^3 collapse in this form would run for hours."""
    cells0 = wr.make_grid(grid)

    def partial(variant):
        c = cells0.copy()
        with wr.Context(len(c), device, math_mode) as ctx:
            if variant is not None:
                ctx.set_variant(variant)
            ctx.upload(c)
            t0 = time.perf_counter()
            cgs, gt, rc = 0, 0.0, wr.SUCCESS
            for step in range(steps):
                rc, dt = ctx.prepare(cgs, gt, step, True)
                if rc != wr.SUCCESS or dt == np.finfo(np.float64).max:
                    break
                rc, cnt = ctx.advance(cgs, gt + dt, dt)
                if rc != wr.SUCCESS or cnt == 0:
                    break
                gt += dt
                cgs += 1
            el = time.perf_counter() - t0
            ctx.download(c)
        return c, el, rc

    ref, t_ref, rc_ref = partial(None)
    c, t_prec, rc = partial(3)
    rT = np.abs(c["T"] - ref["T"]) / ref["T"]
    big = ref["xn"] > 1e-20
    rx = np.abs(c["xn"] - ref["xn"])[big] / ref["xn"][big]
    st, rs = c["stats"], ref["stats"]
    return {
        "workload": f"{grid}^3, first {steps} outer steps", "result": int(rc),
        "cells_steps_per_s": len(c) * steps / t_prec, "plain_fp64_cells_steps_per_s": len(c) * steps / t_ref,
        "vs_plain_fp64_speedup": t_ref / t_prec,
        "attempts_ratio": float(st["internal_steps"].sum()) / max(float(rs["internal_steps"].sum()), 1.0),
        "T_rel_err_max": float(rT.max()), "T_rel_err_median": float(np.median(rT)),
        "species_rel_err_max": float(rx.max()), "species_rel_err_median": float(np.median(rx)),
        "accepted_delta_total": int(st["accepted_steps"].sum()) - int(rs["accepted_steps"].sum()),
        "rejected_delta_total": int((st["internal_steps"] - st["accepted_steps"]).sum())
                                - int((rs["internal_steps"] - rs["accepted_steps"]).sum()),
    }


def cta32_form(wr, device, math_mode, cells0, independent_run_ms, independent_cells, grid, with_reference):
    """The reference's other GPU policy, gridwide-structured-cta32 (one ROS2S
    controller per 32-cell tile), on the bench's own grid: device time of wr_run
    with the state resident (L2 flushed), against the gridwide-independent time and
    final state just measured; cell-attempts and how far the final states differ.
    With ``with_reference``, the reference's own structured kernel on the same grid
    beside it (its time, and whether its final states equal this policy's)."""
    c = cells0.copy()
    with wr.Context(len(c), device, math_mode) as ctx:
        ctx.set_policy(wr.POLICY_GRIDWIDE_CTA32)
        ctx.set_profiling(True)
        ctx.upload(c)
        wr.lib().wr_diag_flush_l2(256)
        rc, cgs = ctx.run(True)
        t = ctx.run_timing()
        ctx.download(c)
    ci = independent_cells
    rT = np.abs(c["T"] / ci["T"] - 1)
    ref = reference_cuda_form(wr, grid, wr.pack_final_states(c, grid), structured=True) if with_reference else None
    return {"workload": "the bench grid, full collapse", "result": int(rc), "reference_structured_kernel": ref,
            "cta32_cells_per_s": len(c) / (t.run_ms / 1e3),
            "independent_cells_per_s": len(c) / (independent_run_ms / 1e3),
            "cta32_over_independent_time": t.run_ms / independent_run_ms,
            "cell_attempts_ratio": float(c["stats"]["internal_steps"].sum()) / float(ci["stats"]["internal_steps"].sum()),
            "T_rel_diff_max": float(rT.max()), "T_rel_diff_median": float(np.median(rT))}


def substeps(cells):
    """ROS2S work summed over cells (IntegratorStats, reproducer.cpp:7433-7441):
    every completed attempt is accepted or rejected, so the exact rejection count
    is attempts - accepted (rejected_steps itself skips rejections before the
    first acceptance, :7337)."""
    st = cells["stats"]
    att, acc = int(st["internal_steps"].sum()), int(st["accepted_steps"].sum())
    return {"attempts": att, "accepted": acc, "rejected_exact": att - acc,
            "rejected_counter": int(st["rejected_steps"].sum()), "jacobians": int(st["jacobian_calls"].sum()),
            "attempts_per_cell": {"min": int(st["internal_steps"].min()),
                                  "median": float(np.median(st["internal_steps"])),
                                  "max": int(st["internal_steps"].max())}}


def error_table(wr, cells, ref):
    """Relative error of ``cells`` against ``ref`` (same grid): T and every species
    above the 1e-20 abundance floor (max and median), and the substep deltas."""
    rT = np.abs(cells["T"] - ref["T"]) / np.abs(ref["T"])
    big = ref["xn"] > 1e-20
    rx = np.abs(cells["xn"] - ref["xn"])[big] / ref["xn"][big]
    per = {}
    for k, name in enumerate(wr.SPECIES):
        b = big[:, k]
        if b.any():
            e = np.abs(cells["xn"][b, k] - ref["xn"][b, k]) / ref["xn"][b, k]
            per[name] = {"max": float(e.max()), "median": float(np.median(e))}
    a, r = substeps(cells), substeps(ref)
    return {"T_rel_err_max": float(rT.max()), "T_rel_err_median": float(np.median(rT)),
            "species_rel_err_max": float(rx.max()) if rx.size else 0.0,
            "species_rel_err_median": float(np.median(rx)) if rx.size else 0.0,
            "per_species": per,
            "attempts_delta": a["attempts"] - r["attempts"], "accepted_delta": a["accepted"] - r["accepted"],
            "rejected_delta": a["rejected_exact"] - r["rejected_exact"]}


def reference_cuda_form(wr, grid, packed_ours, structured=False):
    """The reference's own CUDA kernels (prepare_grid_timestep_kernel and
    advance_collapse_gridwide_kernel, reproducer.cpp:7696-7785, compiled unmodified
    for sm_103a; with ``structured`` its gridwide-structured-cta32 kernel,
    structured_cuda.cuh:393-782) on the same grid and GPU, through the reference's
    host loop (oracle/ref_cuda_launcher.cpp): wall time, cells/s, substep totals,
    and whether its final_states file equals this library's final states (of the
    same policy) byte for byte."""
    import tempfile
    from warp_reactor_gb300 import build
    exe = build.ref_cuda_launcher()
    cubin = os.path.join(ROOT, "oracle", "_ref", "ref_structured.cubin" if structured else "ref_kernels.cubin")
    if not exe or not os.path.exists(cubin):
        return {"unavailable": f"the reference's CUDA kernels were not built ({os.path.relpath(cubin, ROOT)}, made "
                               "where the reference tree exists)"}
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, f"final_states_grid{grid}_cuda.bin")
        r = subprocess.run([exe, cubin, str(grid), out] + (["--structured"] if structured else []),
                           capture_output=True, text=True)
        if r.returncode != 0:
            return {"unavailable": f"launcher exited {r.returncode}: {r.stderr.strip()[-200:]}"}
        line = json.loads(r.stdout.strip().splitlines()[-1])
        ref = np.fromfile(out, wr.PACKED_FINAL_STATE)
    line["kind"] = ("the reference's structured CUDA kernel, one 256-thread block per 32-cell tile, its host loop"
                    if structured else "the reference's CUDA kernels, one thread per cell, 128 per block, its host loop")
    line["final_states_equal_bytes"] = packed_ours.tobytes() == ref.tobytes()
    if not line["final_states_equal_bytes"]:
        rT = np.abs(packed_ours["T"] - ref["T"]) / np.abs(ref["T"])
        line["T_rel_diff_max"] = float(rT.max())
    return line


def portable_form(wr, device, cells0, ref_cells, headline_run_ms):
    """The same collapse with the library's portable exp/log/cbrt (integer pipe, no
    FP64 instructions): its cells/s and its error against the headline run, whose
    final states are the reference CUDA kernel's."""
    c = cells0.copy()
    with wr.Context(len(c), device, wr.MATH_PORTABLE) as ctx:
        ctx.set_profiling(True)
        ctx.upload(c)
        wr.lib().wr_diag_flush_l2(256)
        rc, cgs = ctx.run(True)
        t = ctx.run_timing()
        ctx.download(c)
    out = {"workload": "the bench grid, full collapse, portable exp/log", "result": int(rc),
           "cells_per_s": len(c) / (t.run_ms / 1e3), "over_cuda_math_time": t.run_ms / headline_run_ms}
    out["error_vs_reference"] = error_table(wr, c, ref_cells)
    return out


def diff_measure(grid):
    """Differentiation form (config 4): 16^3 reference cells, perturbations on, the
    plain run's schedule; loss = sum over cells of sum_s w_s (log q_s - log t_s)^2
    over H2, HD, e- and T with a seeded target; gradients in all 15 inputs per cell
    and the network's log rate multipliers (seeded N(0, 0.1^2)).  Times the forward
    map and the adjoint (synchronous calls, best of two).  Gradient checks against
    the FP64 tangent-linear and central differences: tests/test_forms_gpu.py."""
    import torch
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import diff
    cells = wr.make_grid(grid)
    n = len(cells)
    t0 = time.perf_counter()
    sched = diff.schedule(cells)
    plain_s = time.perf_counter() - t0
    rng = np.random.default_rng(2024)
    P = diff.num_multipliers()
    lm = rng.normal(0.0, 0.1, P)
    sel = [8, 10, 0, 14]  # H2, HD, e-, T
    cells_dev = torch.from_numpy(np.ascontiguousarray(cells).view(np.uint8)).cuda()
    u = torch.from_numpy(diff.initial_u(cells)).cuda()
    lm_dev = torch.from_numpy(lm).cuda()
    q = torch.empty((n, 15), dtype=torch.float64, device="cuda")
    with diff.DiffMap(n) as dm:
        fwd, bwd = [], []
        for rep in range(2):
            torch.cuda.synchronize()
            t = time.perf_counter()
            dm.forward(cells_dev, u, lm_dev, sched, True, q)
            fwd.append(time.perf_counter() - t)
            qn = q.cpu().numpy()
            if rep == 0:
                target = qn[:, sel] * np.exp(rng.normal(0.0, 0.1, (n, len(sel))))
            qbar = np.zeros((n, 15))
            qbar[:, sel] = 2.0 * (np.log(qn[:, sel]) - np.log(target)) / qn[:, sel]
            ubar = torch.empty((n, 15), dtype=torch.float64, device="cuda")
            pbar = torch.empty(P, dtype=torch.float64, device="cuda")
            qbar_dev = torch.from_numpy(qbar).cuda()
            torch.cuda.synchronize()
            t = time.perf_counter()
            dm.backward(qbar_dev, ubar, pbar)
            bwd.append(time.perf_counter() - t)
        hbuf, counts = dm.record()
    acc = counts.sum(1)
    loss = float((((np.log(qn[:, sel]) - np.log(target))) ** 2).sum())
    return {
        "form": "differentiation", "grid": grid, "cells": n, "outer_steps": len(sched),
        "multipliers": P, "loss_species": ["H2", "HD", "e-", "T"], "loss": loss,
        "forward_s": min(fwd), "adjoint_s": min(bwd), "adjoint_over_forward": min(bwd) / min(fwd),
        "forward_cells_per_s": n / min(fwd), "plain_run_with_schedule_s": plain_s,
        "accepted_steps_per_cell": {"min": int(acc.min()), "median": float(np.median(acc)), "max": int(acc.max())},
        "checkpoints": "outer-step states (18 doubles per cell per step) + burn checkpoints every 32 accepted steps",
        "grad_norm_u": float(torch.linalg.norm(ubar).item()), "grad_norm_p": float(torch.linalg.norm(pbar).item()),
        "gradient_checks": "tests/test_forms_gpu.py: adjoint vs the FP64 tangent-linear of the same frozen-controller "
                           "map (exact), and vs central differences of that map (replayed step sizes)",
    }


def batch_measure(scale, tune_steps, math_mode):
    """Batching form (config 2): a 128^3 grid plus 32^3, 48^3, 80^3 and 96^3
    sub-grids of the batching workload (seeded log-normal density sigma = 1 dex,
    log-uniform T from 100 K to 10^4 K) in one context: one prepare / order /
    advance launch per outer step covers every cell of every grid, outer steps are
    replayed from a CUDA graph, the launch shape (lanes per cell among them) is
    chosen by the autotuner.  ``scale`` multiplies every grid dimension.  Sampled
    cells of every grid are replayed bit for bit by the oracle in
    tests/test_forms_gpu.py."""
    import warp_reactor_gb300 as wr
    dims = [max(2, int(round(d * scale))) for d in (128, 32, 48, 80, 96)]
    sizes = [d ** 3 for d in dims]
    t = time.perf_counter()
    parts = [wr.make_batch_grid(g, n) for g, n in enumerate(sizes)]
    gen_s = time.perf_counter() - t
    cells = np.concatenate(parts)
    total = len(cells)
    with wr.Context(grids=sizes, math=math_mode) as ctx:
        ctx.upload(cells)
        t = time.perf_counter()
        best = ctx.autotune(True, steps=tune_steps)
        tune_s = time.perf_counter() - t
        ctx.set_profiling(True)
        wr.lib().wr_diag_flush_l2(256)
        t = time.perf_counter()
        rc, cgs = ctx.run(True)
        run_s = time.perf_counter() - t
        timing = ctx.run_timing()
        results = [ctx.grid_result(g) for g in range(len(sizes))]
        ctx.download(cells)
    st = cells["stats"]["internal_steps"]
    return {
        "form": "batching", "scale": scale, "grids": [f"{d}^3" for d in dims], "cells": total, "result": int(rc),
        "cells_per_s": total / (timing.run_ms / 1e3), "run_ms": timing.run_ms, "advance_ms": timing.advance_ms,
        "wall_s": run_s, "autotuned_variant": best, "autotune_s": tune_s, "generate_s": gen_s,
        "grid_results": [list(r) for r in results],
        "attempts_per_cell": {"min": int(st.min()), "median": float(np.median(st)), "max": int(st.max()),
                              "max_over_median": float(st.max() / max(np.median(st), 1))},
        "oracle_checks": "tests/test_forms_gpu.py (sampled cells of every grid, bit for bit)",
    }


def cpu_baseline(grid, threads):
    from oracle import oracle
    o = oracle.load("libm")
    cells = o.make_grid(grid)
    t0 = time.perf_counter()
    rc, cgs = o.run(cells, perturb=True, nthreads=threads)
    dt = time.perf_counter() - t0
    if rc != 1:
        raise RuntimeError(f"CPU oracle failed with {rc}")
    return len(cells) / dt, dt, cgs


def run_reference(args, rank, ws, tdist):
    if rank != 0:
        return 0
    from warp_reactor_gb300 import build
    build.generate_network()
    build.build_oracle()
    threads = os.cpu_count() or 1
    grid = args.ref_grid
    for _ in range(args.warmup):
        cpu_baseline(grid, threads)
    times = []
    n = grid ** 3
    for _ in range(args.steps):
        _, dt, cgs = cpu_baseline(grid, threads)
        times.append(dt)
    total = sum(times)
    value = args.steps * n / total
    line = {
        "impl": "reference", "metric": "cells/s, 64^3 collapse", "value": value, "unit": "cells/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{grid}^3 gridwide-independent full collapse (sample of the 64^3 workload), "
                               "reference CPU arithmetic", "grid": grid, "outer_steps": cgs,
                   "parallelism": f"cpu{threads}"},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                         "sample": f"{grid}^3 full collapse per step, C-library math (bitwise the reference CPU "
                                   f"build), OpenMP over cells"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _profile_figures():
    """Figures of the committed ncu capture of the advance kernel (one launch of the
    64^3 collapse): DRAM bytes per launch and FP64 pipe activity.  Read from
    profiles/, where the capture's command and summary are kept."""
    path = os.path.join(ROOT, "profiles", "k_advance_coop_grid64_traffic.txt")
    out = {}
    if os.path.exists(path):
        for ln in open(path):
            if ":" in ln and not ln.startswith("#"):
                k, v = ln.split(":", 1)
                try:
                    out[k.strip()] = float(v)
                except ValueError:
                    pass
        out["source"] = "profiles/k_advance_coop_grid64_traffic.txt"
    return out


def run_gb300(args, rank, ws, local, tdist):
    t_start = time.perf_counter()
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    math_mode = wr.MATH_CUDA if args.math == "cuda" else wr.MATH_PORTABLE
    grid = args.grid
    cells0 = wr.make_grid(grid)
    n = len(cells0)
    ctx = wr.Context(n, local, math_mode)
    ctx.set_profiling(True)  # event nodes in the graph: per-kernel times of the shipped path
    out = np.empty_like(cells0)

    def one_step():
        ctx.upload(cells0)
        wr.lib().wr_diag_flush_l2(256)
        rc, cgs = ctx.run(True)
        if rc != wr.SUCCESS:
            raise RuntimeError(f"run failed with {rc}: {wr.last_error()}")
        return ctx.run_timing(), cgs

    for _ in range(args.warmup):
        one_step()
    _barrier(tdist)
    launches0 = wr.kernel_launch_count()
    timings = []
    with ClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            t, cgs = one_step()
            timings.append(t)
        t_wall = time.perf_counter() - t_wall
    launches = wr.kernel_launch_count() - launches0
    _barrier(tdist)
    run_s = sum(t.run_ms for t in timings) / 1e3
    value = whole_job_rate(tdist, ws, args.steps, n, run_s)
    run_s = _max_over_ranks(tdist, run_s)
    ctx.download(out)
    adv_ms = sum(t.advance_ms for t in timings)
    adv_launches = sum(t.advance_launches for t in timings)
    ops, opinfo = algorithmic_ops(out)
    peak = wr.fp64_peak()
    achieved = ops * args.steps / (adv_ms / 1e3)
    step_s = run_s / args.steps

    # e2e through the public API with host buffers (timed on the host)
    e2e_cells = cells0.copy()
    _barrier(tdist)
    t0 = time.perf_counter()
    rc, _ = wr.run_cells(e2e_cells, True, math_mode, local)
    e2e_s = _max_over_ranks(tdist, time.perf_counter() - t0)
    if rc != wr.SUCCESS:
        raise RuntimeError(f"e2e run failed with {rc}")
    ctx.close()

    # forms: after the timed region, each only if the wall-clock budget allows
    forms = {}

    def budget_ok(name, est_s):
        if args.forms is not None and name not in args.forms.split(","):
            return False
        left = args.budget_s - (time.perf_counter() - t_start)
        if est_s > left:
            forms[name] = {"skipped": f"wall-clock budget: needs ~{est_s:.0f} s, {left:.0f} s left of --budget-s"}
            return False
        return True

    if not args.no_forms and rank == 0:
        packed = wr.pack_final_states(out, grid)
        if math_mode == wr.MATH_CUDA and budget_ok("reference_cuda_kernel", 70.0):
            forms["reference_cuda_kernel"] = reference_cuda_form(wr, grid, packed)
        if math_mode == wr.MATH_CUDA and budget_ok("portable_math", 1.5 * step_s + 10):
            forms["portable_math"] = portable_form(wr, local, cells0, out, timings[-1].run_ms)
        if budget_ok("cta32_policy", 2.0 * step_s + 100):
            forms["cta32_policy"] = cta32_form(wr, local, math_mode, cells0, timings[-1].run_ms, out, grid,
                                               math_mode == wr.MATH_CUDA)
        if budget_ok("differentiation", 60.0):
            forms["differentiation"] = diff_measure(args.diff_grid)
        if budget_ok("batching", 150.0 * args.forms_batch_scale ** 3 + 30):
            forms["batching"] = batch_measure(args.forms_batch_scale, args.batch_tune_steps, math_mode)
        if budget_ok("precision", 60.0):
            forms["precision"] = precision_form(wr, local, math_mode)
    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt, _ = cpu_baseline(args.cpu_grid, threads)
        cpu = {"value": v, "unit": "cells/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_grid}^3 full collapse ({args.cpu_grid ** 3} cells, {dt:.1f} s), CPU oracle with "
                         f"C-library math (bitwise the reference CPU build), OpenMP over cells"}
    prof = _profile_figures()
    variant_names = {6: "cooperative advance, 16 lanes per cell (generated vector programs, warp-cooperative LU)"}
    line = {
        "metric": "cells/s, 64^3 collapse", "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * run_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / ws / PUBLISHED_CELLS_PER_S if ws == 1 else None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{grid}^3 gridwide-independent collapse, 1000 outer steps, perturbations on, "
                               f"plain FP64, {args.math} exp/log", "grid": grid, "cells": n, "outer_steps": cgs,
                   "form": variant_names.get(6), "path": "wr_run: CUDA-graph replay of 16 outer steps per launch",
                   "l2": "flushed (256 MiB write) before each step", "parallelism": f"replicas{ws}"},
        "substeps": substeps(out),
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12,
                     "unit": "T FP64-op/s (weighted, FMA instruction = 1)", "frac": achieved / peak,
                     "traffic": prof.get("bytes_per_launch"),
                     "peak_source": "measured live: wr_diag_fp64_peak (DFMA chains, all SMs); MEASURED_PEAKS.json "
                                    "has no FP64 figure",
                     "frac_meaning": "algorithm-equivalent: the reference's source-level FP64 work (no CSE, exp/log "
                                     "weighted 25) per second over the FP64 FMA peak",
                     "fp64_pipe_active_ncu": prof.get("fp64_pipe_active"),
                     "profile_source": prof.get("source"),
                     "kernel": "k_advance_coop", "launches": adv_launches,
                     "ms_per_launch": adv_ms / max(adv_launches, 1), "algorithmic_ops_per_step": ops, **opinfo,
                     "programs_per_attempt": program_figures()},
        "cpu_baseline": cpu,
        "e2e": {"value": ws * n / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": n * 216,
                "d2h_bytes_per_step": n * 216},
        "gpu_launches": launches,
        "forms": forms,
        "clocks": clocks.summary(),
        "wall_s_timed": t_wall,
        "wall_s_total": time.perf_counter() - t_start,
    }
    print(json.dumps(line), flush=True)
    return 0


def probe_fp64():
    """FP64 issue interval (cycles per FMA per warp) for 1-16 warps on one SM and
    1/4/8 independent chains per lane, and the whole-GPU FMA rate."""
    import ctypes
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    f = wr.lib().wr_diag_fp64_issue
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    rows = []
    for warps in (1, 2, 4, 8, 16):
        row = {"warps_per_sm": warps}
        for chains in (1, 4, 8):
            v = ctypes.c_double()
            assert f(warps, chains, ctypes.byref(v)) == 1
            row[f"cycles_per_fma_chains{chains}"] = v.value
        rows.append(row)
    print(json.dumps({"fp64_issue": rows, "fp64_fma_per_s": wr.fp64_peak()}), flush=True)
    return 0


def diff_form(args):
    """--diff: the differentiation form alone (see diff_measure)."""
    from warp_reactor_gb300 import build
    build.build_all()
    print(json.dumps(diff_measure(args.diff_grid)), flush=True)
    return 0


def batch_form(args):
    """--batch: the batching form alone (see batch_measure), full size by default."""
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    math_mode = wr.MATH_CUDA if args.math == "cuda" else wr.MATH_PORTABLE
    print(json.dumps(batch_measure(args.batch_scale, args.batch_tune_steps, math_mode)), flush=True)
    return 0


def profile_policy(args):
    """A fixed run for ncu: one full collapse of the grid with the given policy
    through wr_run (``--profile-policy independent|cta32``), printing nothing."""
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    cells = wr.make_grid(args.grid)
    policy = wr.POLICY_GRIDWIDE_CTA32 if args.profile_policy == "cta32" else wr.POLICY_GRIDWIDE_INDEPENDENT
    math_mode = wr.MATH_CUDA if args.math == "cuda" else wr.MATH_PORTABLE
    with wr.Context(len(cells), 0, math_mode) as ctx:
        ctx.set_policy(policy)
        ctx.upload(cells)
        rc, _ = ctx.run(True)
    return 0 if rc == wr.SUCCESS else 1


def profile_phases(args):
    """--profile-phases: one full collapse of the grid through wr_run with the
    cooperative advance's phase counters on (wr_diag_coop_phases): cycles per
    phase of an attempt of one warp, and each phase's share."""
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    cells = wr.make_grid(args.grid)
    math_mode = wr.MATH_CUDA if args.math == "cuda" else wr.MATH_PORTABLE
    with wr.Context(len(cells), 0, math_mode) as ctx:
        if args.variant is not None:
            ctx.set_variant(args.variant)
        ctx.phase_counters(True)
        ctx.set_profiling(True)
        ctx.upload(cells)
        rc, cgs = ctx.run(True)
        t = ctx.run_timing()
        ph = ctx.read_phases()
        ctx.download(cells)
    names = wr.Context.PHASES
    total = sum(ph[k] for k in names)
    print(json.dumps({
        "mode": "profile-phases", "grid": args.grid, "math": args.math, "result": int(rc), "outer_steps": cgs,
        "run_s_with_counters": t.run_ms / 1e3, "warps": ph["warps"], "warp_attempts": ph["attempts"],
        "cycles_per_warp_attempt": {k: ph[k] / max(ph["attempts"], 1) for k in names},
        "share": {k: ph[k] / max(total, 1) for k in names},
        "phase_cycles_over_warp_cycles": total / max(ph["cycles"], 1),
        "cell_attempts": int(cells["stats"]["internal_steps"].sum()),
    }), flush=True)
    return 0 if rc == wr.SUCCESS else 1


def profile_steps(args):
    """A short, fixed run for ncu: ``--profile-steps S`` outer steps of the grid
    through wr_prepare / wr_advance (the same kernels as wr_run)."""
    import warp_reactor_gb300 as wr
    from warp_reactor_gb300 import build
    build.build_all()
    cells = wr.make_grid(args.grid)
    math_mode = wr.MATH_CUDA if args.math == "cuda" else wr.MATH_PORTABLE
    with wr.Context(len(cells), 0, math_mode) as ctx:
        if args.variant is not None:
            ctx.set_variant(args.variant)
        ctx.upload(cells)
        grid_time, done = 0.0, 0
        for step in range(args.profile_steps):
            rc, dt = ctx.prepare(done, grid_time, step, True)
            if rc != wr.SUCCESS or dt == np.finfo(np.float64).max:
                break
            rc, cnt = ctx.advance(done, grid_time + dt, dt)
            if rc != wr.SUCCESS or cnt == 0:
                break
            grid_time += dt
            done += 1
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--math", choices=("cuda", "portable"), default="cuda")
    ap.add_argument("--cpu-grid", type=int, default=16)
    ap.add_argument("--ref-grid", type=int, default=16)
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall-clock budget of the whole run: forms that would exceed it are skipped")
    ap.add_argument("--forms-batch-scale", type=float, default=0.5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the forms after the timed region")
    ap.add_argument("--forms", default=None,
                    help="comma-separated forms to run after the timed region (default: all that fit --budget-s): "
                         "reference_cuda_kernel, portable_math, cta32_policy, differentiation, batching, precision")
    ap.add_argument("--probe-fp64", action="store_true",
                    help="print this GPU's FP64 issue interval per warp count and the FMA peak, exit")
    ap.add_argument("--diff", action="store_true",
                    help="differentiation form: time forward and adjoint on a --diff-grid^3 grid, check gradients")
    ap.add_argument("--diff-grid", type=int, default=16)
    ap.add_argument("--batch", action="store_true",
                    help="batching form: 128^3 + 32^3/48^3/80^3/96^3 sub-grids in one context (see --batch-scale)")
    ap.add_argument("--batch-scale", type=float, default=1.0)
    ap.add_argument("--batch-tune-steps", type=int, default=3)
    ap.add_argument("--profile-policy", choices=("independent", "cta32"), default=None,
                    help="profiling driver: one full collapse with this policy through wr_run, print nothing, exit")
    ap.add_argument("--variant", type=int, default=None,
                    help="advance launch shape of --profile-steps (wr_set_advance_variant; default: the library's)")
    ap.add_argument("--profile-phases", action="store_true",
                    help="diagnostic: one full collapse with the cooperative advance's phase counters, print them, exit")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling driver: run this many outer steps host-stepped, print nothing, exit")
    args = ap.parse_args()
    if args.probe_fp64:
        return probe_fp64()
    if args.diff:
        return diff_form(args)
    if args.batch:
        return batch_form(args)
    if args.profile_policy:
        return profile_policy(args)
    if args.profile_phases:
        return profile_phases(args)
    if args.profile_steps > 0:
        return profile_steps(args)
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    rank, ws, local, tdist = _dist()
    if args.impl == "reference":
        return run_reference(args, rank, ws, tdist)
    return run_gb300(args, rank, ws, local, tdist)


if __name__ == "__main__":
    sys.exit(main())
