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
private subexpressions are computed right before it and their registers die early;
in the fused function the outputs are visited in cone-overlap order
(``overlap_order``).
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


def _cone(dag: Dag, x: int) -> set:
    seen, stack = set(), [x]
    while stack:
        y = stack.pop()
        if y in seen or dag.nodes[y].op in ("const", "in", "bconst"):
            continue
        seen.add(y)
        stack.extend(a for a in dag.nodes[y].args if isinstance(a, int))
    return seen


def overlap_order(dag: Dag, roots) -> list:
    """Output order for the depth-first schedule: repeatedly the output whose
    expression cone is most completely computed already.  Outputs that share
    subexpressions (rate coefficients, common products) then come together, and
    fewer values stay live across the evaluation (peak 419 live values for the
    fused Jacobian + RHS instead of 516 in row order)."""
    outs = list(dict.fromkeys(roots))
    cones = {o: _cone(dag, o) for o in outs}
    order, done, remaining = [], set(), list(outs)
    while remaining:
        best = max(remaining, key=lambda o: (len(cones[o] & done) / (len(cones[o]) + 1), -len(cones[o] - done),
                                            -outs.index(o)))
        order.append(best)
        remaining.remove(best)
        done |= cones[best]
    return order


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


BATCH_OPS = ("exp", "log")
BATCH_MAX = 4
BATCH_WINDOW = 256
# Batched exp/log calls measured slower on GB300 (64^3 collapse: 43.2 s against
# 39.8 s unbatched; the four chains' registers and the hoisted arguments' longer
# live ranges cost more than the latency they hide), so the emitter keeps one call
# per exp/log.  batch_transcendentals stays available behind this switch.
BATCH_TRANSCENDENTALS = False


def batch_transcendentals(dag: Dag, order: list, window: int = BATCH_WINDOW, maxb: int = BATCH_MAX,
                          max_cone: int = 16) -> list:
    """Regroups a schedule so that independent exp (log) nodes are evaluated
    together, up to ``maxb`` per call.  Walking ``order``, at each exp (log) the
    next exp (log) nodes within ``window`` positions join its call when the
    not-yet-computed part of their argument is small (at most ``max_cone`` nodes,
    no exp/log in it); that part is computed first.  The integer-pipe exp/log are
    long dependent instruction chains; four independent chains in one call give
    the SM four times the instruction-level parallelism.  Items: node ids, or
    (op, [ids]) batches, in a valid evaluation order.  Values are unchanged:
    every node is still the same operation on the same operands."""
    leaf = ("const", "in", "bconst")
    pos = {x: i for i, x in enumerate(order)}
    done = set()
    items = []

    def pending_cone(y, group):
        """Not-yet-computed nodes y's argument needs; None when too many or when
        they need a member of the group being formed (computed only after it)."""
        cone, stack = set(), [a for a in dag.nodes[y].args if isinstance(a, int)]
        while stack:
            z = stack.pop()
            if z in group:
                return None
            if z in done or z in cone or dag.nodes[z].op in leaf or z not in pos:
                continue
            cone.add(z)
            if len(cone) > max_cone:
                return None
            stack.extend(a for a in dag.nodes[z].args if isinstance(a, int))
        return cone

    for i, x in enumerate(order):
        if x in done:
            continue
        op = dag.nodes[x].op
        if op not in BATCH_OPS:
            items.append(x)
            done.add(x)
            continue
        group = [x]
        done.add(x)
        for y in order[i + 1:i + 1 + window]:
            if len(group) == maxb:
                break
            if y in done or dag.nodes[y].op != op:
                continue
            cone = pending_cone(y, group)
            if cone is None or any(dag.nodes[z].op in BATCH_OPS for z in cone):
                continue
            for z in sorted(cone, key=pos.get):
                items.append(z)
                done.add(z)
            group.append(y)
            done.add(y)
        items.append(x if len(group) == 1 else (op, group))
    return items


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

    def batch(self, op: str, xs: list):
        """One call evaluating len(xs) independent exp/log nodes."""
        k = len(xs)
        args = ", ".join(self.name(self.dag.nodes[x].args[0]) for x in xs)
        tmp = f"q{xs[0]}"
        self.lines.append(f"    const WrD{k} {tmp} = WrBatch<M>::{op}{k}({args});")
        for j, x in enumerate(xs):
            self.lines.append(f"    const double {self.name(x)} = {tmp}.v{j};")

    def item(self, it):
        if isinstance(it, tuple):
            self.batch(*it)
        else:
            self.node(it)


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
        "// Independent exp/log evaluated together (see emit.py batch_transcendentals).",
        "// WrBatch<M> evaluates them one by one with the policy's exp/log; a policy may",
        "// specialise it with calls that interleave the chains.  Results are identical.",
        "#ifndef WR_BATCH_TYPES",
        "#define WR_BATCH_TYPES",
        "struct WrD2 { double v0, v1; };",
        "struct WrD3 { double v0, v1, v2; };",
        "struct WrD4 { double v0, v1, v2, v3; };",
        "template <class M>",
        "struct WrBatch {",
        "    static WR_NET_HD WrD2 exp2(double a, double b) { return {M::exp(a), M::exp(b)}; }",
        "    static WR_NET_HD WrD3 exp3(double a, double b, double c) { return {M::exp(a), M::exp(b), M::exp(c)}; }",
        "    static WR_NET_HD WrD4 exp4(double a, double b, double c, double d) {",
        "        return {M::exp(a), M::exp(b), M::exp(c), M::exp(d)};",
        "    }",
        "    static WR_NET_HD WrD2 log2(double a, double b) { return {M::log(a), M::log(b)}; }",
        "    static WR_NET_HD WrD3 log3(double a, double b, double c) { return {M::log(a), M::log(b), M::log(c)}; }",
        "    static WR_NET_HD WrD4 log4(double a, double b, double c, double d) {",
        "        return {M::log(a), M::log(b), M::log(c), M::log(d)};",
        "    }",
        "};",
        "#endif",
        "",
    ]
    rhs_roots = dag.rhs_roots()
    jac_roots = dag.jac_roots()

    # RHS only
    w = _Writer(dag)
    rhs_order = schedule(dag, rhs_roots)
    for it in (batch_transcendentals(dag, rhs_order) if BATCH_TRANSCENDENTALS else rhs_order):
        w.item(it)
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_net_rhs(const double* X, const double T, double* f) {")
    out.extend(w.lines)
    for i, r in enumerate(rhs_roots):
        out.append(f"    f[{i}] = {w.name(r)};")
    out.append("}")
    out.append("")

    # fused Jacobian + RHS: schedule J row by row, interleaving outputs as they finish
    w = _Writer(dag)
    fused_order = schedule(dag, overlap_order(dag, jac_roots + rhs_roots))
    items = batch_transcendentals(dag, fused_order) if BATCH_TRANSCENDENTALS else fused_order
    order = []
    for it in items:
        order.append(it)
    emitted_at = {}
    for i, it in enumerate(items):
        for x in (it[1] if isinstance(it, tuple) else [it]):
            emitted_at[x] = i
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
        w.item(x)
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
