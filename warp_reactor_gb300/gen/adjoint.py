"""Derivative code of the network DAG for the differentiation form.

The differentiation form needs, besides the network itself:

* the species/energy RHS with one log multiplier per rate coefficient: every
  rate-coefficient node ``k`` of the RHS is replaced by ``k * mult[r]`` wherever it
  is used (``mult[r] = exp(p[r])``; with ``mult[r] == 1.0`` the product is exactly
  ``k``, so the RHS is bit-for-bit the plain one);
* its vector-Jacobian product (reverse mode): given ``fbar`` (15), the adjoints of
  the inputs ``X`` (14), ``T`` and ``mult`` (accumulated with ``+=``);
* the vector-Jacobian product of the analytic Jacobian (reproducer.cpp:1538-6994)
  with respect to its inputs: given ``Jbar`` (15x15), the adjoints of ``X`` and
  ``T``.  The integrator's iteration matrix ``1/(h gamma) I - J(y)`` depends on the
  state, so the discrete adjoint of a ROS2S step needs it;
* forward-mode (tangent) versions of both, used by the CPU tangent-linear check.

A *rate coefficient* is a node of the RHS that depends on the temperature only, is
not a literal, and is a direct factor of a product term of a species rate
(``k(T) * X_a * X_b``).  Scaling such a node scales every reaction term that
shares it, in every species and in the energy equation, so each multiplier keeps
the network's production/destruction pairs consistent.  The analytic Jacobian is
not rescaled: the integrator keeps the reference's Jacobian of the unscaled network
(at ``mult == 1`` the two coincide); the discrete adjoint differentiates exactly
the map that is computed.

All emitted code is straight-line C++ over a math policy ``M`` (``exp``, ``log``,
``sqrt``, ``fabs``, ``div``), like the network itself.
"""
from __future__ import annotations

from .emit import _Writer, schedule
from .network_dag import Dag

JAC_VJP_CHUNKS = 12


# ----------------------------------------------------------------------------- analysis
def _depends(dag: Dag):
    """Per node: the set of input names it depends on."""
    dep = []
    for n in dag.nodes:
        if n.op == "in":
            dep.append(frozenset((n.args[0],)))
        elif n.op in ("const", "bconst"):
            dep.append(frozenset())
        else:
            s = set()
            for a in n.args:
                s |= dep[a]
            dep.append(frozenset(s))
    return dep


def rate_nodes(dag: Dag) -> list:
    """Rate-coefficient nodes of the species RHS, in node order."""
    dep = _depends(dag)
    nodes = dag.nodes

    def tonly(i):
        return dep[i] <= {"T"}

    def terms(i, out):
        n = nodes[i]
        if n.op in ("add", "sub"):
            terms(n.args[0], out)
            terms(n.args[1], out)
        elif n.op == "neg":
            terms(n.args[0], out)
        else:
            out.append(i)

    def factors(i, out):
        n = nodes[i]
        if n.op == "mul" and not tonly(i):
            factors(n.args[0], out)
            factors(n.args[1], out)
        else:
            out.append(i)

    found = set()
    for s in range(14):
        ts = []
        terms(dag.outputs[("rhs", s)], ts)
        for t in ts:
            fs = []
            factors(t, fs)
            for f in fs:
                if tonly(f) and nodes[f].op not in ("const", "in"):
                    found.add(f)
    return sorted(found)


def multiplied_rhs(dag: Dag):
    """A DAG holding the 15 RHS outputs with every rate node ``k`` replaced by
    ``k * M<r>`` (input node ``M<r>``).  Returns (dag, rate node ids of ``dag``)."""
    rates = rate_nodes(dag)
    slot = {x: r for r, x in enumerate(rates)}
    out = Dag()
    remap = {}
    for x in dag.live_from(dag.rhs_roots()):
        n = dag.nodes[x]
        if n.op in ("const", "bconst", "in"):
            args = n.args
        else:
            args = tuple(remap[a] for a in n.args)
        y = out._intern(n.op, args, n.is_bool)
        if x in slot:
            m = out._intern("in", (f"M{slot[x]}",))
            y = out._intern("mul", (y, m))
        remap[x] = y
    for i in range(15):
        out.outputs[("rhs", i)] = remap[dag.outputs[("rhs", i)]]
    return out, rates


# ----------------------------------------------------------------------------- writers
class _AdjWriter(_Writer):
    """Writer that also names the multiplier inputs ``M<r>`` as ``mult[r]``."""

    def name(self, x: int) -> str:
        n = self.dag.nodes[x]
        if n.op == "in" and n.args[0].startswith("M"):
            return f"mult[{n.args[0][1:]}]"
        return super().name(x)


def _active(dag: Dag, order):
    act = set()
    for x in order:
        n = dag.nodes[x]
        if n.is_bool or n.op in ("const", "bconst", "cexp", "clog", "csqrt", "b2d"):
            continue
        if n.op == "in":
            act.add(x)
            continue
        args = n.args[1:] if n.op == "sel" else n.args
        if any(a in act for a in args):
            act.add(x)
    return act


def _input_ref(dag: Dag, x: int, kind: str) -> str:
    """Adjoint (``kind='bar'``) or tangent (``kind='d'``) of an input node."""
    nm = dag.nodes[x].args[0]
    if nm == "T":
        return "Tbar" if kind == "bar" else "dT"
    if nm.startswith("M"):
        return f"mbar[{nm[1:]}]" if kind == "bar" else f"dmult[{nm[1:]}]"
    return f"Xbar[{nm[1:]}]" if kind == "bar" else f"dX[{nm[1:]}]"


def _vjp_body(dag: Dag, roots, seed_names) -> list:
    """Forward sweep plus reverse sweep.  ``seed_names[i]`` is the C expression of
    the adjoint of ``roots[i]``."""
    w = _AdjWriter(dag)
    order = schedule(dag, roots)
    for x in order:
        w.node(x)
    lines = list(w.lines)
    act = _active(dag, order)
    declared = set()
    body = []

    def acc(x, expr):
        if x not in act:
            return
        n = dag.nodes[x]
        if n.op == "in":
            body.append(f"    {_input_ref(dag, x, 'bar')} += {expr};")
            return
        if x in declared:
            body.append(f"    a{x} += {expr};")
        else:
            declared.add(x)
            body.append(f"    double a{x} = {expr};")

    for r, s in zip(roots, seed_names):
        acc(r, s)
    nm = w.name
    for x in reversed(order):
        if x not in act or x not in declared:
            continue
        n = dag.nodes[x]
        op, a = n.op, n.args
        g = f"a{x}"
        if op == "add":
            acc(a[0], g)
            acc(a[1], g)
        elif op == "sub":
            acc(a[0], g)
            acc(a[1], f"-{g}")
        elif op == "mul":
            acc(a[0], f"WR_AMUL({g}, {nm(a[1])})")
            acc(a[1], f"WR_AMUL({g}, {nm(a[0])})")
        elif op == "div":
            acc(a[0], f"WR_ADIV({g}, {nm(a[1])})")
            acc(a[1], f"-WR_ADIV(WR_AMUL({g}, {nm(x)}), {nm(a[1])})")
        elif op == "neg":
            acc(a[0], f"-{g}")
        elif op == "abs":
            acc(a[0], f"({nm(a[0])} < 0.0 ? -{g} : {g})")
        elif op == "exp":
            acc(a[0], f"WR_AMUL({g}, {nm(x)})")
        elif op == "log":
            acc(a[0], f"WR_ADIV({g}, {nm(a[0])})")
        elif op == "sqrt":
            acc(a[0], f"WR_ADIV(0.5 * {g}, {nm(x)})")
        elif op == "sel":
            acc(a[1], f"({nm(a[0])} ? {g} : 0.0)")
            acc(a[2], f"({nm(a[0])} ? 0.0 : {g})")
        elif op == "in":
            pass
        else:
            raise ValueError(f"no derivative rule for {op}")
    return lines + body


def _vjp_chunked(dag: Dag, roots, seed_names, name: str, sig: str, chunks: int) -> list:
    """Reverse mode split into ``chunks`` out-of-line functions.

    A single straight-line function of the Jacobian's size (~20k statements) takes
    ptxas minutes to compile; chunks of a few hundred nodes compile in seconds.
    The schedule is cut into contiguous chunks.  Forward chunk k computes its
    nodes and stores the values that later chunks read into ``V`` (one slot per
    cross-chunk value); reverse chunk k recomputes its own nodes (reading earlier
    chunks' values from ``V``), then propagates adjoints in reverse order: within
    the chunk in registers, to earlier chunks through ``A`` (same slots), to the
    inputs into ``Xbar``/``Tbar``.  The J forward pass is thus evaluated twice;
    the live state between chunks is the slot arrays instead of register spills.
    """
    order = schedule(dag, roots)
    act = _active(dag, order)
    leaf = ("const", "in", "bconst")
    body_nodes = [x for x in order if dag.nodes[x].op not in leaf]
    size = (len(body_nodes) + chunks - 1) // chunks
    chunk_of = {x: i // size for i, x in enumerate(body_nodes)}
    nchunks = max(chunk_of.values()) + 1
    slot = {}
    for x in body_nodes:
        for a in dag.nodes[x].args:
            if isinstance(a, int) and a in chunk_of and chunk_of[a] < chunk_of[x] and a not in slot:
                slot[a] = len(slot)
    nslots = max(len(slot), 1)
    seeds = {}
    for r, sname in zip(roots, seed_names):
        seeds.setdefault(r, []).append(sname)

    class W(_AdjWriter):
        def __init__(self, dag, k):
            super().__init__(dag)
            self.k = k

        def name(self, x):
            if x in chunk_of and chunk_of[x] != self.k:
                return f"(V[{slot[x]}] != 0.0)" if dag.nodes[x].is_bool else f"V[{slot[x]}]"
            return super().name(x)

    funcs = []
    # forward chunks
    for k in range(nchunks):
        w = W(dag, k)
        for x in body_nodes:
            if chunk_of[x] == k:
                w.node(x)
        lines = list(w.lines)
        for x in body_nodes:
            if chunk_of[x] == k and x in slot:
                v = f"(b{x} ? 1.0 : 0.0)" if dag.nodes[x].is_bool else f"v{x}"
                lines.append(f"    V[{slot[x]}] = {v};")
        funcs.append(("template <class M>",
                      f"WR_NET_CHUNK void {name}_f{k}(const double* X, const double T, double* V) {{",
                      lines))
    # reverse chunks
    touched = set()
    for k in reversed(range(nchunks)):
        w = W(dag, k)
        mine = [x for x in body_nodes if chunk_of[x] == k]
        for x in mine:
            w.node(x)
        lines = list(w.lines)
        declared = set()
        nm = w.name

        def acc(x, expr):
            if x not in act:
                return
            n = dag.nodes[x]
            if n.op == "in":
                lines.append(f"    {_input_ref(dag, x, 'bar')} += {expr};")
                return
            if chunk_of[x] == k:
                if x in declared:
                    lines.append(f"    a{x} += {expr};")
                else:
                    declared.add(x)
                    lines.append(f"    double a{x} = {expr};")
            else:
                if x in touched:
                    lines.append(f"    A[{slot[x]}] += {expr};")
                else:
                    touched.add(x)
                    lines.append(f"    A[{slot[x]}] = {expr};")

        for x in mine:
            if x in touched:
                declared.add(x)
                lines.append(f"    double a{x} = A[{slot[x]}];")
        for x in mine:
            for sname in seeds.get(x, []):
                acc(x, sname)
        for x in reversed(mine):
            if x not in act or x not in declared:
                continue
            n = dag.nodes[x]
            op, a = n.op, n.args
            g = f"a{x}"
            if op == "add":
                acc(a[0], g)
                acc(a[1], g)
            elif op == "sub":
                acc(a[0], g)
                acc(a[1], f"-{g}")
            elif op == "mul":
                acc(a[0], f"WR_AMUL({g}, {nm(a[1])})")
                acc(a[1], f"WR_AMUL({g}, {nm(a[0])})")
            elif op == "div":
                acc(a[0], f"WR_ADIV({g}, {nm(a[1])})")
                acc(a[1], f"-WR_ADIV(WR_AMUL({g}, {nm(x)}), {nm(a[1])})")
            elif op == "neg":
                acc(a[0], f"-{g}")
            elif op == "abs":
                acc(a[0], f"({nm(a[0])} < 0.0 ? -{g} : {g})")
            elif op == "exp":
                acc(a[0], f"WR_AMUL({g}, {nm(x)})")
            elif op == "log":
                acc(a[0], f"WR_ADIV({g}, {nm(a[0])})")
            elif op == "sqrt":
                acc(a[0], f"WR_ADIV(0.5 * {g}, {nm(x)})")
            elif op == "sel":
                acc(a[1], f"({nm(a[0])} ? {g} : 0.0)")
                acc(a[2], f"({nm(a[0])} ? 0.0 : {g})")
            else:
                raise ValueError(f"no derivative rule for {op}")
        funcs.append(("template <class M>",
                      f"WR_NET_CHUNK void {name}_r{k}(const double* X, const double T, {sig}, const double* V,"
                      " double* A, double* Xbar, double& Tbar) {", lines))
    # roots that are inputs directly (no chunk) still take their seeds
    tail = []
    for r, sname in zip(roots, seed_names):
        if dag.nodes[r].op == "in" and r in act:
            tail.append(f"    {_input_ref(dag, r, 'bar')} += {sname};")
    up = name.upper()
    out = [f"#define {up}_CHUNKS {nchunks}", f"#define {up}_SLOTS {nslots}", ""]
    for head, decl, lines in funcs:
        out.append(head)
        out.append(decl)
        out.extend(lines)
        out.append("}")
        out.append("")
    out.append("template <class M>")
    out.append(f"WR_NET_HD void {name}(const double* X, const double T, {sig}, double* Xbar, double& Tbar) {{")
    out.append(f"    double V[{up}_SLOTS], A[{up}_SLOTS];")
    for k in range(nchunks):
        out.append(f"    {name}_f{k}<M>(X, T, V);")
    argname = sig.split()[-1].lstrip("*")
    for k in reversed(range(nchunks)):
        out.append(f"    {name}_r{k}<M>(X, T, {argname}, V, A, Xbar, Tbar);")
    out.extend(tail)
    out.append("}")
    out.append("")
    return out


def _jvp_body(dag: Dag, roots):
    """Forward sweep with tangents; returns (lines, tangent name of node)."""
    w = _AdjWriter(dag)
    order = schedule(dag, roots)
    act = _active(dag, order)
    nm = w.name
    tan = {}
    lines = []

    def t(x):
        return tan.get(x)

    for x in order:
        before = len(w.lines)
        w.node(x)
        lines.extend(w.lines[before:])
        if x not in act:
            continue
        n = dag.nodes[x]
        op, a = n.op, n.args
        if op == "in":
            tan[x] = _input_ref(dag, x, "d")
            continue
        ta = [t(v) for v in a]
        if op == "add":
            e = " + ".join(p for p in ta if p)
        elif op == "sub":
            if ta[0] and ta[1]:
                e = f"{ta[0]} - {ta[1]}"
            elif ta[0]:
                e = ta[0]
            else:
                e = f"-{ta[1]}"
        elif op == "mul":
            parts = []
            if ta[0]:
                parts.append(f"{ta[0]} * {nm(a[1])}")
            if ta[1]:
                parts.append(f"{nm(a[0])} * {ta[1]}")
            e = " + ".join(parts)
        elif op == "div":
            if ta[0] and ta[1]:
                e = f"M::div({ta[0]} - {nm(x)} * {ta[1]}, {nm(a[1])})"
            elif ta[0]:
                e = f"M::div({ta[0]}, {nm(a[1])})"
            else:
                e = f"-M::div({nm(x)} * {ta[1]}, {nm(a[1])})"
        elif op == "neg":
            e = f"-{ta[0]}"
        elif op == "abs":
            e = f"({nm(a[0])} < 0.0 ? -{ta[0]} : {ta[0]})"
        elif op == "exp":
            e = f"{nm(x)} * {ta[0]}"
        elif op == "log":
            e = f"M::div({ta[0]}, {nm(a[0])})"
        elif op == "sqrt":
            e = f"M::div(0.5 * {ta[0]}, {nm(x)})"
        elif op == "sel":
            e = f"({nm(a[0])} ? {ta[1] or '0.0'} : {ta[2] or '0.0'})"
        else:
            raise ValueError(f"no derivative rule for {op}")
        tan[x] = f"t{x}"
        lines.append(f"    const double t{x} = {e};")
    return lines, (lambda x: tan.get(x) or "0.0"), nm


# ----------------------------------------------------------------------------- header
def emit_header(dag: Dag, ir_digest: str) -> str:
    mdag, rates = multiplied_rhs(dag)
    nrates = len(rates)
    rhs_roots = mdag.rhs_roots()
    jac_roots = dag.jac_roots()
    out = [
        "// Generated by warp_reactor_gb300/gen/adjoint.py from network.ir",
        f"// network.ir sha256 {ir_digest}",
        "// Do not edit: regenerate with `python -m warp_reactor_gb300.gen.build_network`.",
        "#pragma once",
        "#ifndef WR_NET_HD",
        "#define WR_NET_HD inline",
        "#endif",
        "",
        "// Reverse-mode products that stay 0 when the adjoint is 0: the branch a select",
        "// did not take may hold inf or NaN values, and 0 * inf must not leak into the",
        "// inputs' adjoints.",
        "#define WR_AMUL(g, x) (((g) == 0.0) ? 0.0 : (g) * (x))",
        "#define WR_ADIV(g, x) (((g) == 0.0) ? 0.0 : M::div((g), (x)))",
        "",
        f"#define WR_NUM_RATE_MULT {nrates}",
        "",
        "// network.ir node ids of the rate coefficients, multiplier order",
        "static const int wr_rate_node_ids[WR_NUM_RATE_MULT] = {"
        + ", ".join(str(x) for x in rates) + "};",
        "",
    ]
    # forward RHS with multipliers
    w = _AdjWriter(mdag)
    for x in schedule(mdag, rhs_roots):
        w.node(x)
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_netp_rhs(const double* X, const double T, const double* mult, double* f) {")
    out.extend(w.lines)
    for i, r in enumerate(rhs_roots):
        out.append(f"    f[{i}] = {w.name(r)};")
    out.append("}")
    out.append("")
    # RHS VJP
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_netp_rhs_vjp(const double* X, const double T, const double* mult,"
               " const double* fbar, double* Xbar, double& Tbar, double* mbar) {")
    out.extend(_vjp_body(mdag, rhs_roots, [f"fbar[{i}]" for i in range(15)]))
    out.append("}")
    out.append("")
    # J VJP, in out-of-line chunks (see _vjp_chunked)
    out.append("#ifndef WR_NET_CHUNK")
    out.append("#define WR_NET_CHUNK inline")
    out.append("#endif")
    out.extend(_vjp_chunked(dag, jac_roots, [f"Jbar[{r * 15 + c}]" for r in range(15) for c in range(15)],
                            "wr_net_jac_vjp", "const double* Jbar", JAC_VJP_CHUNKS))
    # RHS JVP
    lines, tan, nm = _jvp_body(mdag, rhs_roots)
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_netp_rhs_jvp(const double* X, const double T, const double* mult,"
               " const double* dX, const double dT, const double* dmult, double* f, double* df) {")
    out.extend(lines)
    for i, r in enumerate(rhs_roots):
        out.append(f"    f[{i}] = {nm(r)};")
        out.append(f"    df[{i}] = {tan(r)};")
    out.append("}")
    out.append("")
    # J JVP
    lines, tan, nm = _jvp_body(dag, jac_roots)
    out.append("template <class M>")
    out.append("WR_NET_HD void wr_net_jac_jvp(const double* X, const double T, const double* dX,"
               " const double dT, double* J, double* dJ) {")
    out.extend(lines)
    for r in range(15):
        for c in range(15):
            x = dag.outputs[("jac", r, c)]
            out.append(f"    J[{r * 15 + c}] = {nm(x)};")
            out.append(f"    dJ[{r * 15 + c}] = {tan(x)};")
    out.append("}")
    out.append("")
    return "\n".join(out) + "\n"
