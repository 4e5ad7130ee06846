"""Write the golden fixtures of tests/golden/ from the reference itself.

Run where the reference tree is present, after ``oracle/build_ref.sh`` has built
``oracle/_ref/libwr_ref.so`` (the reference's reproducer.cpp compiled from its own
sources with a C shim) and ``oracle/_ref/reproducer_cpu`` (the unmodified
reference program):

    python tests/golden/make_golden.py

Fixtures (all values produced by the reference's own code):
  network_ref.npz      actual_rhs / actual_jac at the initial state with
                       T = 10, 100, 1e4, 3e4 K (the reference's slice-DAG test
                       states, tests/test_slice_dag.mojo:88-92) and at 256 seeded
                       random burn states
  lu_ref.npz           lu_decomposition / lu_solve on the eight matrices of the
                       reference's LU test (tests/gpu/test_warp_lu.mojo:19-47)
  grids_ref.npz        CollapseState of every cell after the gridwide-independent
                       run at grid 1, 2, 3, 4 (perturbations on) and grid 2
                       (perturbations off), with the completed global steps
  grid1_stdout_ref.txt the reference CPU program's output for --grid 1
  legacy_grid{2,3}_ref.bin  final_states_grid<N>_cpu.bin written by the reference
                       CPU program (its default legacy-local policy) for --grid 2, 3
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402


def lu_case(case_id):
    """The reference LU test matrices (tests/gpu/test_warp_lu.mojo:19-47)."""
    A = np.zeros((15, 15))
    b = np.zeros(15)
    for r in range(15):
        for c in range(15):
            if case_id <= 3:
                v = 1.0 if r == c else 0.0
            else:
                v = float((r * 17 + c * 13 + case_id * 7) % 19 - 9) * 0.01
                if r == c:
                    v += 2.0
            A[r, c] = v
        b[r] = float((r * 5 + case_id * 3) % 11 - 5)
    if case_id == 1:
        A[14, :] = 0.0
    elif case_id == 2:
        A[0, 0] = 0.0
        A[1, 0] = 2.0
    elif case_id == 3:
        A[0, 0] = 1.0
        A[1, 0] = -3.0
        A[2, 0] = 3.0
    elif case_id == 7:
        A[14, 14] = 1.0e-10
    return A, b


def random_states(n, seed=20261203):
    rng = np.random.default_rng(seed)
    X = 10.0 ** rng.uniform(-40, 18, size=(n, 14))
    T = 10.0 ** rng.uniform(0.5, 5.0, size=n)
    return X, T


def main():
    ref = orc.load("ref")
    init = ref.make_collapse_state()
    Xs, Ts = [], []
    for T in (10.0, 100.0, 1.0e4, 3.0e4):
        Xs.append(np.array(init["xn"]))
        Ts.append(T)
    Xr, Tr = random_states(256)
    X = np.vstack([np.array(Xs), Xr])
    T = np.concatenate([np.array(Ts), Tr])
    J = np.zeros((len(T), 15, 15))
    F = np.zeros((len(T), 15))
    for i in range(len(T)):
        J[i], _ = ref.net_jac(X[i], T[i])
        F[i] = ref.net_rhs(X[i], T[i])
    np.savez_compressed(os.path.join(HERE, "network_ref.npz"), X=X, T=T, J=J, f=F)

    As, bs, LUs, ips, infos, xs = [], [], [], [], [], []
    for case in range(8):
        A, b = lu_case(case)
        info, LU, ip = ref.lu(A)
        x = ref.lu_solve(LU, ip, b) if info == 0 else b.copy()
        As.append(A); bs.append(b); LUs.append(LU); ips.append(ip); infos.append(info); xs.append(x)
    np.savez_compressed(os.path.join(HERE, "lu_ref.npz"), A=np.array(As), b=np.array(bs), LU=np.array(LUs),
                        ipvt=np.array(ips), info=np.array(infos), x=np.array(xs))

    out = {}
    for grid, perturb in ((1, True), (2, True), (3, True), (4, True), (2, False)):
        cells = ref.make_grid(grid)
        rc, cgs = ref.run(cells, perturb=perturb, nthreads=os.cpu_count())
        assert rc == 1, rc
        key = f"grid{grid}_{'p' if perturb else 'np'}"
        out[key + "_cells"] = cells
        out[key + "_cgs"] = np.int32(cgs)
    np.savez_compressed(os.path.join(HERE, "grids_ref.npz"), **out)

    exe = os.path.join(ROOT, "oracle", "_ref", "reproducer_cpu")
    r = subprocess.run([exe, "--grid", "1", "--no-compare-final-state"], capture_output=True, text=True, check=True)
    lines = [ln for ln in r.stdout.splitlines() if not ln.startswith("wall time")]
    with open(os.path.join(HERE, "grid1_stdout_ref.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    import shutil
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        for g in (2, 3):
            subprocess.run([exe, "--grid", str(g), "--no-compare-final-state"], capture_output=True, text=True,
                           check=True, cwd=tmp)
            shutil.copy(os.path.join(tmp, f"final_states_grid{g}_cpu.bin"), os.path.join(HERE, f"legacy_grid{g}_ref.bin"))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
