"""Read the reference's generated network code into a :class:`network_dag.Dag`.

The reference ships its RHS and analytic Jacobian as machine-generated straight-line
C++ (``rhs_specie`` reproducer.cpp:342-677, ``rhs_eint`` :679-1512, ``jac_nuc``
:1538-6994).  This module is a small C++-expression parser for exactly that subset:

* statements ``Real xN = e;``, ``xN = e;``, ``ydot(k) = e;``, ``jac(r,c) = e;`` and
  ``return e;`` (the energy rate);
* expressions with literals, ``X(i)``, ``T``, ``z``, temporaries, ``+ - * /``, unary
  ``- + !``, comparisons, ``&& ||``, ``?:`` and ``std::exp/log/sqrt/abs/fabs``;
* C++ typing where it matters: integer literals stay ``int`` until they meet a
  ``double`` (so ``1/2`` would be 0), comparisons are ``bool``, and a ``bool`` stored
  into a ``Real`` temporary is 0.0/1.0 (used again as a condition it is the same
  predicate).

Operator precedence and left-to-right associativity follow C++, so ``a*b*c`` is
``(a*b)*c``: the DAG computes the reference's rounding sequence.

This module reads the reference tree and therefore runs only where that tree is
present; its output is stored with ``ir_io.save`` and committed.
"""
from __future__ import annotations

import re

from .network_dag import Dag, OP_WEIGHT

_TOKEN = re.compile(
    r"\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?)"
    r"|(?P<id>[A-Za-z_][A-Za-z_0-9]*(?:::[A-Za-z_][A-Za-z_0-9]*)*)"
    r"|(?P<op><=|>=|==|!=|&&|\|\||[-+*/()<>?:!,;=]))"
)


def tokenize(text: str):
    pos = 0
    out = []
    text = text.rstrip()
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            raise SyntaxError(f"bad token at {text[pos:pos + 40]!r}")
        pos = m.end()
        if m.group("num") is not None:
            out.append(("num", m.group("num")))
        elif m.group("id") is not None:
            out.append(("id", m.group("id")))
        else:
            out.append(("op", m.group("op")))
    return out


_MATH_MACROS = {
    "M_LN10": "2.30258509299404568402",
    "M_PI": "3.14159265358979323846",
}


class _Val:
    """A typed expression value: kind is 'int', 'real' or 'bool'."""

    __slots__ = ("kind", "node", "ival", "cost")

    def __init__(self, kind, node=None, ival=None, cost=None):
        self.kind = kind
        self.node = node
        self.ival = ival
        self.cost = cost or {}


def _merge(*costs):
    out = {}
    for c in costs:
        for k, v in c.items():
            out[k] = out.get(k, 0) + v
    return out


class _Parser:
    def __init__(self, dag: Dag, env: dict, toks):
        self.dag = dag
        self.env = env  # name -> _Val (temporaries carry zero source cost)
        self.toks = toks
        self.i = 0

    # ------------------------------------------------------------ token helpers
    def peek(self, k=0):
        j = self.i + k
        return self.toks[j] if j < len(self.toks) else ("eof", None)

    def take(self, expect=None):
        t = self.peek()
        if expect is not None and t[1] != expect:
            raise SyntaxError(f"expected {expect!r}, got {t!r}")
        self.i += 1
        return t

    # ------------------------------------------------------------ conversions
    def real(self, v: _Val) -> int:
        d = self.dag
        if v.kind == "real":
            return v.node
        if v.kind == "int":
            return d.const(float(v.ival))
        return d.unary("b2d", v.node)

    def boolean(self, v: _Val) -> int:
        d = self.dag
        if v.kind == "bool":
            return v.node
        if v.kind == "int":
            return d.binary("ne", d.const(float(v.ival)), d.const(0.0))
        n = d.nodes[v.node]
        if n.op == "b2d":
            return n.args[0]
        return d.binary("ne", v.node, d.const(0.0))

    # ------------------------------------------------------------ grammar
    def expr(self) -> _Val:
        return self.ternary()

    def ternary(self) -> _Val:
        c = self.lor()
        if self.peek()[1] == "?":
            self.take("?")
            a = self.expr()
            self.take(":")
            b = self.ternary()
            # an int-valued ternary is represented by its (exact) double value
            if a.kind == "bool" and b.kind == "bool":
                node = self.dag.bselect(self.boolean(c), a.node, b.node)
                big = a.cost if self.dag.weighted(a.cost) >= self.dag.weighted(b.cost) else b.cost
                return _Val("bool", node, cost=_merge(c.cost, big))
            node = self.dag.select(self.boolean(c), self.real(a), self.real(b))
            # source cost: the reference evaluates the condition and one branch;
            # count the larger branch (an upper bound used only for reporting)
            big = a.cost if self.dag.weighted(a.cost) >= self.dag.weighted(b.cost) else b.cost
            return _Val("real", node, cost=_merge(c.cost, big))
        return c

    def lor(self) -> _Val:
        v = self.land()
        while self.peek()[1] == "||":
            self.take()
            w = self.land()
            v = _Val("bool", self.dag.binary("or", self.boolean(v), self.boolean(w)),
                     cost=_merge(v.cost, w.cost))
        return v

    def land(self) -> _Val:
        v = self.equality()
        while self.peek()[1] == "&&":
            self.take()
            w = self.equality()
            v = _Val("bool", self.dag.binary("and", self.boolean(v), self.boolean(w)),
                     cost=_merge(v.cost, w.cost))
        return v

    def equality(self) -> _Val:
        v = self.relational()
        while self.peek()[1] in ("==", "!="):
            op = {"==": "eq", "!=": "ne"}[self.take()[1]]
            w = self.relational()
            v = _Val("bool", self.dag.binary(op, self.real(v), self.real(w)),
                     cost=_merge(v.cost, w.cost))
        return v

    def relational(self) -> _Val:
        v = self.additive()
        while self.peek()[1] in ("<", "<=", ">", ">="):
            op = {"<": "lt", "<=": "le", ">": "gt", ">=": "ge"}[self.take()[1]]
            w = self.additive()
            v = _Val("bool", self.dag.binary(op, self.real(v), self.real(w)),
                     cost=_merge(v.cost, w.cost))
        return v

    def _arith(self, op, v: _Val, w: _Val) -> _Val:
        if v.kind == "int" and w.kind == "int":
            a, b = v.ival, w.ival
            if op == "add":
                r = a + b
            elif op == "sub":
                r = a - b
            elif op == "mul":
                r = a * b
            else:
                q = abs(a) // abs(b)
                r = q if (a >= 0) == (b >= 0) else -q
            return _Val("int", ival=r)
        node = self.dag.binary(op, self.real(v), self.real(w))
        return _Val("real", node, cost=_merge(v.cost, w.cost, {op: 1}))

    def _powi(self, n: int, x: int):
        """integrators::math::powi<n>(x) exactly as reproducer.cpp:64-72 recurses."""
        d = self.dag
        if n < 0:
            p, c = self._powi(-n, x)
            return d.binary("div", d.const(1.0), p), _merge(c, {"div": 1})
        if n == 0:
            return d.const(1.0), {}
        if n == 1:
            return x, {}
        if n == 2:
            return d.binary("mul", x, x), {"mul": 1}
        if n % 2 == 0:
            p, c = self._powi(n // 2, x)
            return d.binary("mul", p, p), _merge(c, {"mul": 1})
        p, c = self._powi(n - 1, x)
        return d.binary("mul", x, p), _merge(c, {"mul": 1})

    def additive(self) -> _Val:
        v = self.multiplicative()
        while self.peek()[1] in ("+", "-"):
            op = "add" if self.take()[1] == "+" else "sub"
            v = self._arith(op, v, self.multiplicative())
        return v

    def multiplicative(self) -> _Val:
        v = self.unary()
        while self.peek()[1] in ("*", "/"):
            op = "mul" if self.take()[1] == "*" else "div"
            v = self._arith(op, v, self.unary())
        return v

    def unary(self) -> _Val:
        t = self.peek()
        if t[1] == "-":
            self.take()
            v = self.unary()
            if v.kind == "int":
                return _Val("int", ival=-v.ival)
            return _Val("real", self.dag.neg(self.real(v)), cost=v.cost)
        if t[1] == "+":
            self.take()
            return self.unary()
        if t[1] == "!":
            self.take()
            v = self.unary()
            return _Val("bool", self.dag.unary("not", self.boolean(v)), cost=v.cost)
        return self.primary()

    def primary(self) -> _Val:
        t = self.take()
        kind, text = t
        if kind == "num":
            if re.fullmatch(r"\d+", text):
                return _Val("int", ival=int(text))
            return _Val("real", self.dag.const(float(text)))
        if kind == "op" and text == "(":
            v = self.expr()
            self.take(")")
            return v
        if kind == "id":
            if text in ("std::exp", "std::log", "std::sqrt", "std::abs", "std::fabs"):
                self.take("(")
                a = self.expr()
                self.take(")")
                fn = text.split("::")[1]
                if fn == "abs" and a.kind == "int":
                    return _Val("int", ival=abs(a.ival))
                op = "abs" if fn in ("abs", "fabs") else fn
                node = self.dag.unary(op, self.real(a))
                src = {} if a.kind == "int" or self.dag.nodes[self.real(a)].op == "const" else {op: 1}
                return _Val("real", node, cost=_merge(a.cost, src))
            if text == "integrators::math::powi":
                # powi<N>(x), reproducer.cpp:64-72
                self.take("<")
                sign = 1
                if self.peek()[1] == "-":
                    self.take()
                    sign = -1
                n = sign * int(self.take()[1])
                self.take(">")
                self.take("(")
                a = self.expr()
                self.take(")")
                node, cost = self._powi(n, self.real(a))
                return _Val("real", node, cost=_merge(a.cost, cost))
            if text == "X":
                self.take("(")
                idx = self.expr()
                self.take(")")
                assert idx.kind == "int"
                return _Val("real", self.dag.inp(f"X{idx.ival}"))
            if text in ("T", "z"):
                return _Val("real", self.dag.inp(text))
            if text in ("true", "false"):
                return _Val("bool", self.dag.bconst(text == "true"))
            if text in _MATH_MACROS:
                # <cmath> macros expand to decimal literals; parsing them rounds as
                # the compiler does
                return _Val("real", self.dag.const(float(_MATH_MACROS[text])))
            if text in self.env:
                v = self.env[text]
                return _Val(v.kind, v.node, v.ival, cost={})
        raise SyntaxError(f"unexpected token {t!r}")


def _statements(body: str):
    """Split a function body into ';'-terminated statements (comments removed)."""
    body = re.sub(r"//[^\n]*", "", body)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    for stmt in body.split(";"):
        stmt = " ".join(stmt.split())
        if stmt:
            yield stmt


def _body(lines, start, end):
    """Text between the first '{' at/after line ``start`` and the matching '}'."""
    text = "\n".join(lines[start - 1:end])
    i = text.index("{")
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[i + 1:j]
    raise SyntaxError("unbalanced body")


_ASSIGN = re.compile(r"^(?:Real\s+)?(?P<lhs>x\d+|T|ydot\(\d+\)|jac\(\d+,\d+\))\s*=\s*(?P<rhs>.*)$")


def _run_function(dag: Dag, body: str, sink):
    env = {}
    for stmt in _statements(body):
        if stmt.startswith("return "):
            p = _Parser(dag, env, tokenize(stmt[len("return "):]))
            v = p.expr()
            assert p.peek()[0] == "eof"
            sink("return", v, p)
            continue
        m = _ASSIGN.match(stmt)
        if not m:
            raise SyntaxError(f"unsupported statement: {stmt[:80]!r}")
        lhs, rhs = m.group("lhs"), m.group("rhs")
        if lhs == "T":
            assert rhs == "state.T", rhs
            continue
        p = _Parser(dag, env, tokenize(rhs))
        v = p.expr()
        if p.peek()[0] != "eof":
            raise SyntaxError(f"trailing tokens in {stmt[:80]!r}")
        if lhs.startswith("x"):
            # a temporary: remember its value and the source-level cost of defining it
            v.cost = dict(v.cost)
            env[lhs] = v
            sink("temp", v, p)
        else:
            sink(lhs, v, p)


def extract(path: str) -> Dag:
    """Parse the reference file at ``path`` into a DAG with 15 RHS and 225 J outputs.

    The generated expressions nest deeply, so parsing runs on a thread with a large
    stack and a raised recursion limit.
    """
    import sys
    import threading

    result = {}

    def work():
        try:
            result["dag"] = _extract(path)
        except BaseException as exc:  # re-raised on the calling thread
            result["err"] = exc

    old_limit = sys.getrecursionlimit()
    old_stack = threading.stack_size()
    sys.setrecursionlimit(200000)
    threading.stack_size(512 * 1024 * 1024)
    try:
        t = threading.Thread(target=work)
        t.start()
        t.join()
    finally:
        threading.stack_size(old_stack)
        sys.setrecursionlimit(old_limit)
    if "err" in result:
        raise result["err"]
    return result["dag"]


def _extract(path: str) -> Dag:
    with open(path) as f:
        text = f.read()
    lines = text.split("\n")

    def find(sig):
        for n, line in enumerate(lines, 1):
            if sig in line:
                return n
        raise KeyError(sig)

    dag = Dag()
    src = {"rhs": {}, "jac": {}}

    def account(group, v, p):
        for k, c in v.cost.items():
            src[group][k] = src[group].get(k, 0) + c

    # rhs_specie: ydot(1..14) -> species rates 0..13
    def sink_species(kind, v, p):
        account("rhs", v, p)
        if kind.startswith("ydot("):
            k = int(kind[5:-1])
            dag.outputs[("rhs", k - 1)] = p.real(v)

    start = find("void rhs_specie(const burn_t& state,")
    _run_function(dag, _body(lines, start, start + 400), sink_species)

    def sink_eint(kind, v, p):
        account("rhs", v, p)
        if kind == "return":
            dag.outputs[("rhs", 14)] = p.real(v)

    start = find("Real rhs_eint(const burn_t& state,")
    _run_function(dag, _body(lines, start, start + 900), sink_eint)

    def sink_jac(kind, v, p):
        account("jac", v, p)
        if kind.startswith("jac("):
            r, c = (int(s) for s in kind[4:-1].split(","))
            dag.outputs[("jac", r - 1, c - 1)] = p.real(v)

    start = find("void jac_nuc(const burn_t& state,")
    end = find("void actual_jac(const burn_t& state, MatrixType& jac)")
    _run_function(dag, _body(lines, start, end), sink_jac)

    for i in range(15):
        dag.outputs.setdefault(("rhs", i), dag.const(0.0))
    for r in range(15):
        for c in range(15):
            dag.outputs.setdefault(("jac", r, c), dag.const(0.0))
    dag.source_counts = src
    return dag
