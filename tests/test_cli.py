"""The drop-in reproducer program: arguments, exit codes, files, comparator."""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def exe(built):
    return built["cli"]


def run(exe, *args, cwd=None):
    return subprocess.run([exe, *args], capture_output=True, text=True, cwd=cwd, timeout=600)


def test_help_and_usage(exe):
    r = run(exe, "--help")
    assert r.returncode == 0 and "usage:" in r.stderr
    for bad in (["--grid"], ["--grid", "0"], ["--grid", "-3"], ["--grid", "x"], ["--bogus"],
                ["--compare-final-state"], ["--compare-final-state="], ["--math", "fast"]):
        r = run(exe, *bad)
        assert r.returncode == 1 and "usage:" in r.stderr, bad
        assert "PASS" not in r.stdout and "FAIL" not in r.stdout


def test_grid_too_large(exe):
    r = run(exe, "--grid", "2000")
    assert r.returncode == 1 and "grid dimension is too large: 2000" in r.stderr


def _parse(stdout):
    return dict(ln.split(": ", 1) for ln in stdout.splitlines() if ": " in ln)


@pytest.mark.gpu
def test_grid1_prints_state(exe, gpu, oracle_port):
    r = run(exe, "--grid", "1", "--math", "portable")
    assert r.returncode == 0, r.stderr
    v = _parse(r.stdout)
    assert v["driver policy"] == "gridwide-independent"
    cells = oracle_port.make_grid(1)
    rc, cgs = oracle_port.run(cells, perturb=True)
    assert int(v["completed global collapse steps"]) == cgs
    assert float(v["T"]) == float(cells["T"][0])  # printed with 17 significant digits
    assert int(v["ROS2S internal steps"]) == int(cells["stats"]["internal_steps"][0])
    assert "PASS" not in r.stdout  # no comparison requested


@pytest.mark.gpu
def test_grid2_file_rotation_and_compare(exe, gpu, tmp_path, oracle_port, wr):
    r = run(exe, "--grid", "2", "--math", "portable", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    f = tmp_path / "final_states_grid2_cuda.bin"
    assert f.stat().st_size == 8 * 172
    got = np.fromfile(f, wr.PACKED_FINAL_STATE)
    cells = oracle_port.make_grid(2)
    oracle_port.run(cells, perturb=True)
    assert got.tobytes() == wr.pack_final_states(cells, 2).tobytes()
    # second run rotates the file and compares against the first: PASS, exit 0
    r = run(exe, "--grid", "2", "--math", "portable", "--compare-final-state", str(f), cwd=tmp_path)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("PASS"), r.stdout
    assert "existing final states moved to:" in r.stdout
    assert len(list(tmp_path.glob("final_states_grid2_cuda.bin.old.*"))) == 1
    # a perturbed reference file fails with a CSV of the failing fields
    bad = got.copy()
    bad["T"][3] *= 1.01
    bad["completed_steps"][5] += 1
    badf = tmp_path / "bad.bin"
    bad.tofile(badf)
    r = run(exe, "--grid", "2", "--math", "portable", f"--compare-final-state={badf}", cwd=tmp_path)
    assert r.returncode == 1 and r.stdout.rstrip().endswith("FAIL")
    assert "first comparison failure: metadata mismatch at cell 3" not in r.stdout
    csv = (tmp_path / "final_state_comparison_failures_cuda.csv").read_text().splitlines()
    assert csv[0] == "cell,i,j,k,field,actual,reference,relative_error,rtol,atol"
    fields = {(ln.split(",")[0], ln.split(",")[4]) for ln in csv[1:]}
    assert ("3", "T") in fields and ("5", "completed_steps") in fields
    # wrong-size file: read error, FAIL
    r = run(exe, "--grid", "2", "--compare-final-state", str(tmp_path / "missing.bin"), cwd=tmp_path)
    assert r.returncode == 1 and "failed to open final-state comparison file" in r.stderr


@pytest.mark.gpu
def test_default_math_equals_reference_cuda_kernel(exe, gpu, tmp_path, wr):
    """With no --math the program computes in CUDA math and writes the final
    states of the reference's own CUDA build (reproducer.cpp compiled with nvcc
    for sm_103a, run on GB300) byte for byte, and the comparator passes on them."""
    ref = os.path.join(os.path.dirname(__file__), "golden", "refcuda_grid4.bin")
    r = run(exe, "--grid", "4", "--compare-final-state", ref, cwd=tmp_path)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("PASS"), r.stdout
    got = (tmp_path / "final_states_grid4_cuda.bin").read_bytes()
    assert got == open(ref, "rb").read()


def test_policy_and_write_flags_parse(exe):
    for bad in (["--driver-policy"], ["--driver-policy", "cta64"], ["--write-final-state"]):
        r = run(exe, *bad)
        assert r.returncode == 1 and "usage:" in r.stderr, bad
    r = run(exe, "--help")
    assert "gridwide-independent|legacy-local|gridwide-cta32" in (r.stdout + r.stderr)


@pytest.mark.gpu
def test_legacy_local_cli_and_manifest(exe, gpu, tmp_path, oracle_port, wr):
    out = tmp_path / "legacy.bin"
    r = run(exe, "--grid", "2", "--math", "portable", "--driver-policy", "legacy-local",
            "--write-final-state", str(out), cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "driver policy: legacy-local" in r.stdout
    cells = oracle_port.make_grid(2)
    oracle_port.run_legacy(cells, perturb=True)
    assert out.read_bytes() == wr.pack_final_states(cells, 2).tobytes()
    man = (tmp_path / "legacy.bin.manifest").read_text()
    assert "policy=legacy-local-v1" in man and "cell_count=8" in man
    r = run(exe, "--grid", "2", "--write-final-state", str(out), cwd=tmp_path)
    assert r.returncode == 1 and "refusing to overwrite" in r.stderr


@pytest.mark.gpu
def test_cta32_cli(exe, gpu, tmp_path, oracle_port, wr):
    """--driver-policy gridwide-cta32 prints the reference structured build's policy
    name and writes the tile-controller final states."""
    out = tmp_path / "cta32.bin"
    r = run(exe, "--grid", "2", "--math", "portable", "--driver-policy", "gridwide-cta32",
            "--write-final-state", str(out), cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "driver policy: gridwide-structured-cta32" in r.stdout
    cells = oracle_port.make_grid(2)
    oracle_port.run_cta32(cells, perturb=True)
    assert out.read_bytes() == wr.pack_final_states(cells, 2).tobytes()
    assert "policy=gridwide-cta32-v1" in (tmp_path / "cta32.bin.manifest").read_text()
