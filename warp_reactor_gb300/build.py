"""Build recipe: generated network header, the CUDA library, the CLI and the oracle.

All outputs are written in-tree and git-ignored:

  warp_reactor_gb300/csrc/generated/network_gen.h   emitted from gen/network.ir
  warp_reactor_gb300/_build/libwarp_reactor.so       the C-ABI library (sm_103a)
  warp_reactor_gb300/_build/reproducer_gb300         the drop-in CLI
  oracle/_build/libwr_oracle_port.so                 CPU oracle, portable math
  oracle/_build/libwr_oracle_libm.so                 CPU oracle, C-library math
  oracle/_build/libwr_oracle_prec.so                 CPU oracle, the precision form's arithmetic

Translation units compile in parallel; a unit is rebuilt only when one of its
inputs is newer than its object.  No cmake: nvcc and g++ are driven directly.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_OUT = os.path.join(ORACLE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: a*b+c stays two roundings, the reference's operation sequence.
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC"]

CUDA_UNITS = ["wr_capi.cu", "wr_adv_portable.cu", "wr_adv_cuda.cu", "wr_adv_cta32.cu", "wr_diag.cu", "wr_noalloc.cu",
              "wr_adv_coop8.cu", "wr_adv_coop16.cu", "wr_adv_coop32.cu"]
# differentiation form: relocatable device code, device-linked into one object
# (its generated derivative code is split over several units that compile in parallel)
RDC_UNITS = ["wr_diff.cu", "wr_diff_bwd.cu", "wr_diff_net.cu", "wr_diff_jvjp0.cu", "wr_diff_jvjp1.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build warp_reactor_gb300")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd, verbose=False, env=None):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def generate_network() -> str:
    from .gen import build_network
    return build_network.emit_header()


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(CSRC, "generated", "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def build_library(verbose=False, jobs=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    objs = []
    tasks = []
    rdc_objs = []
    for unit in CUDA_UNITS + RDC_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        rdc = unit in RDC_UNITS
        (rdc_objs if rdc else objs).append(obj)
        if _stale(obj, [src] + headers):
            tasks.append([nvcc] + NVCC_FLAGS + (["-rdc=true"] if rdc else []) + ["-c", src, "-o", obj])
    # longest units first
    tasks.sort(key=lambda c: 0 if any(u in c[-3] for u in ("jvjp", "bwd", "net")) else 1)
    with cf.ThreadPoolExecutor(max_workers=jobs or len(CUDA_UNITS) + len(RDC_UNITS)) as ex:
        list(ex.map(lambda c: _run(c, verbose), tasks))
    dlink = os.path.join(OUT, "wr_diff_dlink.o")
    if _stale(dlink, rdc_objs):
        _run([nvcc] + ARCH + ["-dlink", "-Xcompiler", "-fPIC", "-o", dlink] + rdc_objs, verbose)
    lib = os.path.join(OUT, "libwarp_reactor.so")
    all_objs = objs + rdc_objs + [dlink]
    if _stale(lib, all_objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + all_objs + ["-lcudart"], verbose)
    return lib


def build_cli(verbose=False) -> str:
    src = os.path.join(CSRC, "reproducer_main.cpp")
    exe = os.path.join(OUT, "reproducer_gb300")
    lib = os.path.join(OUT, "libwarp_reactor.so")
    if not os.path.exists(src):
        return ""
    if _stale(exe, [src, lib, os.path.join(INCLUDE, "warp_reactor.h")]):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", INCLUDE, "-o", exe, src,
              "-L", OUT, "-lwarp_reactor", "-Wl,-rpath,$ORIGIN"], verbose)
    return exe


def build_oracle(verbose=False) -> list:
    """Compile the CPU oracle (test infrastructure) in both math modes."""
    os.makedirs(ORACLE_OUT, exist_ok=True)
    src = os.path.join(ORACLE, "wr_oracle.cpp")
    deps = [src, os.path.join(CSRC, "wr_math.h"), os.path.join(CSRC, "wr_math_tables.h"),
            os.path.join(CSRC, "generated", "network_gen.h"), os.path.join(INCLUDE, "warp_reactor.h")]
    outs = []
    tasks = []
    for name, defs in (("libwr_oracle_port.so", []), ("libwr_oracle_libm.so", ["-DWR_ORACLE_LIBM"]),
                       ("libwr_oracle_prec.so", ["-DWR_ORACLE_PREC=2"])):
        so = os.path.join(ORACLE_OUT, name)
        outs.append(so)
        if _stale(so, deps):
            tasks.append(["g++"] + CXX_FLAGS + ["-fopenmp", "-shared"] + defs + ["-o", so, src])
    # the differentiation form's map and tangent-linear (portable math)
    dsrc = os.path.join(ORACLE, "wr_oracle_diff.cpp")
    dso = os.path.join(ORACLE_OUT, "libwr_oracle_diff.so")
    outs.append(dso)
    if _stale(dso, deps + [dsrc, os.path.join(CSRC, "generated", "network_adj.h")]):
        tasks.append(["g++"] + CXX_FLAGS + ["-fopenmp", "-shared", "-o", dso, dsrc])
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(lambda c: _run(c, verbose), tasks))
    ref_cuda_launcher(verbose)
    return outs


def ref_cuda_launcher(verbose=False) -> str:
    """Compile the host launcher of the reference's own CUDA kernels (test and
    benchmark infrastructure: it runs oracle/_ref/ref_kernels.cubin through the
    reference's host loop).  Returns its path, or "" where the CUDA driver library
    stub is missing."""
    src = os.path.join(ORACLE, "ref_cuda_launcher.cpp")
    exe = os.path.join(ORACLE_OUT, "ref_cuda_launcher")
    home = _cuda_home()
    stubs = [d for d in (os.path.join(home, "lib64", "stubs"), os.path.join(home, "targets", "sbsa-linux", "lib", "stubs"),
                         os.path.join(home, "targets", "x86_64-linux", "lib", "stubs")) if os.path.isdir(d)]
    if not os.path.exists(src) or not stubs:
        return ""
    os.makedirs(ORACLE_OUT, exist_ok=True)
    if _stale(exe, [src, os.path.join(INCLUDE, "warp_reactor.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I", os.path.join(home, "include"), "-o", exe, src] +
             [f"-L{d}" for d in stubs] + ["-lcuda"], verbose)
    return exe


def build_reference_oracle(verbose=False) -> None:
    """Compile the reference itself into oracle/_ref (only where its tree exists)."""
    script = os.path.join(ORACLE, "build_ref.sh")
    # REF_DIR names the reference checkout; by default its sibling of this repository
    ref_dir = os.environ.get("REF_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
    ref_src = os.path.join(ref_dir, "reproducer.cpp")
    if not (os.path.exists(ref_src) and os.path.exists(script)):
        return
    deps = [ref_src, script, os.path.join(ORACLE, "ref_shim.cpp"), os.path.join(INCLUDE, "warp_reactor.h")]
    cuda_deps = [ref_src, script, os.path.join(ORACLE, "ref_cuda_shim.cu")]
    # The reference's CUDA kernels (plain and structured) are device code: built
    # here, they travel with the repository to a GPU host that has no reference tree.
    env = dict(os.environ, WITH_CUBIN="1", WITH_STRUCTURED="1", PATH=os.path.dirname(_nvcc()) + os.pathsep +
               os.environ.get("PATH", ""))
    stale = _stale(os.path.join(ORACLE, "_ref", "libwr_ref.so"), deps)
    for name in ("ref_kernels.cubin", "ref_structured.cubin"):
        stale = stale or _stale(os.path.join(ORACLE, "_ref", name), cuda_deps)
    if stale:
        _run(["sh", script], verbose, env=env)


def build_all(verbose=False) -> dict:
    generate_network()
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle, verbose)
        f_ref = ex.submit(build_reference_oracle, verbose)
        lib = f_lib.result()
        oracle = f_orc.result()
        f_ref.result()
    cli = build_cli(verbose)
    return {"library": lib, "cli": cli, "oracle": oracle}


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
