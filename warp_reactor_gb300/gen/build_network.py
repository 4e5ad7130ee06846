"""Generator entry point: reference text -> ``network.ir`` -> emitted C++ header.

``python -m warp_reactor_gb300.gen.build_network extract <reproducer.cpp>``
    parses the reference's generated RHS/Jacobian code into the DAG and rewrites
    ``network.ir`` (needs the reference tree; run once, the IR is committed);

``python -m warp_reactor_gb300.gen.build_network emit [out.h]``
    writes ``csrc/generated/network_gen.h`` and ``csrc/generated/network_adj.h``
    (derivative code, ``adjoint.py``) from the committed ``network.ir`` (run by
    the package build on every machine);

``python -m warp_reactor_gb300.gen.build_network counts``
    prints the source-level and CSE'd operation counts.
"""
from __future__ import annotations

import os
import sys

from . import adjoint as _adjoint
from . import emit as _emit
from . import ir_io

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_HEADER = os.path.join(os.path.dirname(HERE), "csrc", "generated", "network_gen.h")
ADJOINT_HEADER = os.path.join(os.path.dirname(HERE), "csrc", "generated", "network_adj.h")

IR_HEADER = """\
14-species primordial network (H/He/D, energy equation), RHS and analytic Jacobian.
Parsed by warp_reactor_gb300/gen/extract.py from the reference's generated code
(reproducer.cpp rhs_specie :342-677, rhs_eint :679-1512, jac_nuc :1538-6994), with
exact-arithmetic CSE, commutative operand ordering, sign normalisation and constant
folding (z = 30).  Inputs: X0..X13 number densities (floored), T temperature."""


def op_counts(dag):
    rhs = dag.count(dag.rhs_roots())
    jac = dag.count(dag.jac_roots())
    both = dag.count(dag.rhs_roots() + dag.jac_roots())
    return {
        "source_rhs": dag.source_counts.get("rhs", {}),
        "source_jac": dag.source_counts.get("jac", {}),
        "source_rhs_weighted": dag.weighted(dag.source_counts.get("rhs", {})),
        "source_jac_weighted": dag.weighted(dag.source_counts.get("jac", {})),
        "cse_rhs": rhs,
        "cse_jac": jac,
        "cse_jac_rhs": both,
        "cse_rhs_weighted": dag.weighted(rhs),
        "cse_jac_weighted": dag.weighted(jac),
        "cse_jac_rhs_weighted": dag.weighted(both),
    }


def _write_if_changed(path: str, text: str) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    old = None
    if os.path.exists(path):
        with open(path) as f:
            old = f.read()
    if old != text:
        with open(path, "w") as f:
            f.write(text)


def emit_header(out_path: str = DEFAULT_HEADER, ir_path: str = ir_io.DEFAULT_PATH,
                adjoint_path: str = ADJOINT_HEADER) -> str:
    """Write the network header and, beside it, the derivative code of the
    differentiation form (``network_adj.h``)."""
    dag = ir_io.load(ir_path)
    digest = ir_io.digest(ir_path)
    _write_if_changed(out_path, _emit.emit_header(dag, digest))
    _write_if_changed(adjoint_path, _adjoint.emit_header(dag, digest))
    from . import coop as _coop
    _coop.emit_all(os.path.dirname(out_path), ir_path)
    return out_path


def main(argv):
    if not argv or argv[0] not in ("extract", "emit", "counts"):
        print(__doc__)
        return 2
    if argv[0] == "extract":
        from .extract import extract
        dag = extract(argv[1])
        digest = ir_io.save(dag, header=IR_HEADER)
        print("network.ir written, sha256", digest)
        return 0
    if argv[0] == "emit":
        print(emit_header(*(argv[1:2] or [DEFAULT_HEADER])))
        return 0
    dag = ir_io.load()
    for k, v in op_counts(dag).items():
        print(k, v)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
