#!/usr/bin/env python3
"""Time the reference's own CPU program as it is: a reported-only baseline.

``oracle/_ref/reproducer_cpu`` is the unmodified reference program
(reproducer.cpp, built by oracle/build_ref.sh with ``c++ -O3``).  Its CPU build
runs the legacy-local policy single-threaded (reproducer.cpp:7646-7685, the host
loop of :8591-8660).  This script runs it at the given grids in a temporary
directory (it writes final_states_grid<N>_cpu.bin there) with
``--no-compare-final-state`` and prints one JSON line per grid: process wall time,
cells/s, the completed global steps and the ROS2S counters it prints.

It runs only where oracle/_ref was built (a machine with the reference tree); the
host's CPU model and the thread count (1) are part of the line.

    python oracle/time_reference_cpu.py [--grids 1,4,8]
"""
import argparse
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "_ref", "reproducer_cpu")


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def run(grid: int) -> dict:
    with tempfile.TemporaryDirectory() as tmp:
        t0 = time.perf_counter()
        r = subprocess.run([EXE, "--grid", str(grid), "--no-compare-final-state"], cwd=tmp,
                           capture_output=True, text=True)
        wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(f"reproducer_cpu --grid {grid} exited {r.returncode}: {r.stderr[-500:]}")
    out = r.stdout

    def field(name):
        m = re.search(rf"^{re.escape(name)}:\s*(.+)$", out, re.M)
        return m.group(1).strip() if m else None

    cells = grid ** 3
    return {"program": "reference reproducer (CPU build, unmodified)", "policy": "legacy-local",
            "grid": grid, "cells": cells, "wall_s": wall, "cells_per_s": cells / wall, "threads": 1,
            "cpu": cpu_model(), "completed_global_steps": field("completed global collapse steps"),
            "internal_steps": field("ROS2S internal steps"), "accepted_rejected": field("ROS2S accepted/rejected")}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--grids", default="1,4,8")
    args = ap.parse_args()
    if not os.path.exists(EXE):
        print(json.dumps({"unavailable": f"{os.path.relpath(EXE)} not built (oracle/build_ref.sh needs the "
                                         f"reference tree)"}))
        return 0
    for g in (int(x) for x in args.grids.split(",")):
        print(json.dumps(run(g)), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
