"""Emit the network DAG as C++ usable from host code and from CUDA device code.

The emitted header defines two function templates over a math policy ``M``:

``wr_net_rhs<M>(const double* X, double T, double* f)``
    the 15 right-hand-side values (14 species rates, then the energy rate), i.e.
    ``actual_rhs`` (reproducer.cpp:1515-1535) without the adapter;

``wr_net_jac_rhs<M>(const double* X, double T, double* f, S& sink)``
    the same 15 values plus the 225 Jacobian entries, delivered as
    ``sink(row, col, value)`` with 0-based row/col (``jac_nuc`` uses 1-based
    ``jac(row, col)``, reproducer.cpp:7014-7020).  Sharing the DAG between the
    Jacobian and the RHS at the same state is exact: identical operations on
    identical operands.

The policy supplies ``M::exp, M::log, M::sqrt, M::fabs`` and ``M::div``; every other
operation is a plain binary64 ``+ - *`` or a comparison, written in the DAG's
(reference) operand order.  The host and device builds must not contract ``a*b+c``
into an FMA (``-ffp-contract=off`` / ``--fmad=false``) for the results to be the
reference's rounding sequence.

Emission order: a depth-first schedule from the outputs, so that each output's
private subexpressions are computed right before it and their registers die early.
"""
from __future__ import annotations

from .network_dag import Dag


def _fmt_const(hexval: str) -> str:
    v = float.fromhex(hexval)
    if v != v:
        return "(0.0/0.0)"
    if v in (float("inf"), float("-inf")):
        return "(1.0/0.0)" if v > 0 else "(-1.0/0.0)"
    r = repr(v)
    if "e" not in r and "." not in r and "inf" not in r:
        r += ".0"
    return r


def schedule(dag: Dag, roots) -> list:
    """Depth-first post-order of the nodes reachable from ``roots`` (roots in order)."""
    order = []
    seen = set()
    for root in roots:
        stack = [(root, False)]
        while stack:
            x, expanded = stack.pop()
            if x in seen:
                continue
            n = dag.nodes[x]
            if expanded or n.op in ("const", "in", "bconst"):
                seen.add(x)
                order.append(x)
                continue
            stack.append((x, True))
            for a in reversed(n.args):
                if a not in seen:
                    stack.append((a, False))
    return order


class _Writer:
    def __init__(self, dag: Dag):
        self.dag = dag
        self.lines = []

    def name(self, x: int) -> str:
        n = self.dag.nodes[x]
        if n.op == "const":
            return _fmt_const(n.args[0])
        if n.op == "bconst":
            return "true" if n.args[0] else "false"
        if n.op == "in":
            nm = n.args[0]
            return "T" if nm == "T" else f"X[{nm[1:]}]"
        return ("b" if n.is_bool else "v") + str(x)

    def node(self, x: int):
        n = self.dag.nodes[x]
        op, a = n.op, n.args
        if op in ("const", "in", "bconst"):
            return
        nm = self.name
        if op == "add":
            e = f"{nm(a[0])} + {nm(a[1])}"
        elif op == "sub":
            e = f"{nm(a[0])} - {nm(a[1])}"
        elif op == "mul":
            e = f"{nm(a[0])} * {nm(a[1])}"
        elif op == "div":
            e = f"M::div({nm(a[0])}, {nm(a[1])})"
        elif op == "neg":
            e = f"-{nm(a[0])}"
        elif op == "abs":
            e = f"M::fabs({nm(a[0])})"
        elif op in ("exp", "cexp"):
            e = f"M::exp({nm(a[0])})"
        elif op in ("log", "clog"):
            e = f"M::log({nm(a[0])})"
        elif op in ("sqrt", "csqrt"):
            e = f"M::sqrt({nm(a[0])})"
        elif op == "le":
            e = f"{nm(a[0])} <= {nm(a[1])}"
        elif op == "lt":
            e = f"{nm(a[0])} < {nm(a[1])}"
        elif op == "eq":
            e = f"{nm(a[0])} == {nm(a[1])}"
        elif op == "ne":
            e = f"{nm(a[0])} != {nm(a[1])}"
        elif op == "and":
            e = f"{nm(a[0])} && {nm(a[1])}"
        elif op == "or":
            e = f"{nm(a[0])} || {nm(a[1])}"
        elif op == "not":
            e = f"!{nm(a[0])}"
        elif op == "b2d":
            e = f"({nm(a[0])} ? 1.0 : 0.0)"
        elif op == "sel":
            e = f"{nm(a[0])} ? {nm(a[1])} : {nm(a[2])}"
        else:
            raise ValueError(op)
        ty = "bool" if n.is_bool else "double"
        self.lines.append(f"    const {ty} {nm(x)} = {e};")


def emit_header(dag: Dag, ir_digest: str) -> str:
    out = [
        "// Generated by warp_reactor_gb300/gen/emit.py from network.ir",
        f"// network.ir sha256 {ir_digest}",
        "// Do not edit: regenerate with `python -m warp_reactor_gb300.gen.build_network`.",
        "#pragma once",
        "#ifndef WR_NET_HD",
        "#define WR_NET_HD inline",
        "#endif",
        "",
    ]
    rhs_roots = dag.rhs_roots()
    jac_roots = dag.jac_roots()

    # RHS only
    w = _Writer(dag)
    for x in schedule(dag, rhs_roots):
        w.node(x)
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_net_rhs(const double* X, const double T, double* f) {")
    out.extend(w.lines)
    for i, r in enumerate(rhs_roots):
        out.append(f"    f[{i}] = {w.name(r)};")
    out.append("}")
    out.append("")

    # fused Jacobian + RHS: schedule J row by row, interleaving outputs as they finish
    w = _Writer(dag)
    order = schedule(dag, jac_roots + rhs_roots)
    emitted_at = {x: i for i, x in enumerate(order)}
    pending = []
    for r in range(15):
        for c in range(15):
            pending.append((emitted_at[dag.outputs[("jac", r, c)]], f"    sink({r}, {c}, {{}});",
                            dag.outputs[("jac", r, c)]))
    for i in range(15):
        pending.append((emitted_at[dag.outputs[("rhs", i)]], f"    f[{i}] = {{}};",
                        dag.outputs[("rhs", i)]))
    pending.sort(key=lambda t: t[0])
    pi = 0
    body = []
    for k, x in enumerate(order):
        before = len(w.lines)
        w.node(x)
        body.extend(w.lines[before:])
        while pi < len(pending) and pending[pi][0] <= k:
            body.append(pending[pi][1].format(w.name(pending[pi][2])))
            pi += 1
    while pi < len(pending):
        body.append(pending[pi][1].format(w.name(pending[pi][2])))
        pi += 1
    out.append("template <class M, class S>")
    out.append("WR_NET_HD void wr_net_jac_rhs(const double* X, const double T, double* f, S& sink) {")
    out.extend(body)
    out.append("}")
    out.append("")
    return "\n".join(out) + "\n"
