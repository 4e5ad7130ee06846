"""Expression-DAG model of the 14-species primordial network (RHS + analytic Jacobian).

The chemistry network is data: 14 species rates, one energy rate and 225 Jacobian
entries, each an expression of the 14 number densities X(0..13), the temperature T
and the redshift z.  This module holds that data as a hash-consed DAG whose
simplifications are all exact in IEEE binary64 round-to-nearest arithmetic, so that
any schedule of the DAG computes bit-for-bit the values that the reference's
straight-line generated code computes (reproducer.cpp:342-1512 for the RHS,
reproducer.cpp:1538-6994 for the Jacobian):

* common-subexpression elimination (the same operation on the same operands gives
  the same value);
* operand ordering of the commutative ``add`` / ``mul`` (IEEE ``a+b == b+a`` and
  ``a*b == b*a`` exactly);
* sign normalisation: ``(-a)*b -> -(a*b)``, ``a+(-b) -> a-b`` ... (negation commutes
  with correctly rounded ``+ - * /`` under round-to-nearest);
* constant folding of ``+ - * /`` on literals (Python floats are binary64 RN, the same
  arithmetic the compiler folds with), with the redshift z fixed to 30
  (reproducer.cpp:219-225 returns 30 on the device; the host sets 30 in ``main``).

Transcendentals of constants (``log(10.0)``, ``sqrt(10)``) are kept as ``cexp`` /
``clog`` / ``csqrt`` nodes so that each emitter decides how to evaluate them.

Reassociation, distribution and reciprocal tricks are *not* applied: they change
rounding.  The module has no dependency on the reference tree; ``extract.py`` builds a
DAG from the reference text once and ``ir_io.py`` stores it under this package.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

# Weighted operation cost used for the algorithmic FLOP count.  exp/log = 25 and
# sqrt/cbrt = 20, each + - * / = 1 (the reference's slicer cost model,
# tools/slice_dag.py:297-302).  Compares, selects and sign/abs changes cost 0.
OP_WEIGHT = {
    "add": 1, "sub": 1, "mul": 1, "div": 1,
    "exp": 25, "log": 25, "sqrt": 20,
    "neg": 0, "abs": 0, "sel": 0, "le": 0, "lt": 0, "ge": 0, "gt": 0,
    "eq": 0, "ne": 0, "and": 0, "or": 0, "not": 0, "b2d": 0,
    "const": 0, "bconst": 0, "in": 0, "cexp": 0, "clog": 0, "csqrt": 0,
}

BOOL_OPS = {"le", "lt", "ge", "gt", "eq", "ne", "and", "or", "not"}
COMMUTATIVE = {"add", "mul", "eq", "ne", "and", "or"}

INPUT_NAMES = tuple([f"X{i}" for i in range(14)] + ["T"])
REDSHIFT = 30.0


@dataclass
class Node:
    op: str
    args: tuple  # node ids, or a float for "const", or a name for "in"
    is_bool: bool = False


@dataclass
class Dag:
    nodes: list = field(default_factory=list)
    index: dict = field(default_factory=dict)
    # named outputs: ("rhs", i) for i in 0..14, ("jac", r, c) for r, c in 0..14
    outputs: dict = field(default_factory=dict)
    # source-level (pre-CSE) weighted op counts per output group, recorded by the parser
    source_counts: dict = field(default_factory=dict)

    # ---------------------------------------------------------------- construction
    def _intern(self, op: str, args: tuple, is_bool: bool = False) -> int:
        key = (op, args)
        nid = self.index.get(key)
        if nid is None:
            nid = len(self.nodes)
            self.nodes.append(Node(op, args, is_bool))
            self.index[key] = nid
        return nid

    def const(self, value: float) -> int:
        value = float(value)
        # +0.0 and -0.0 are distinct constants; key on the bit pattern via repr
        return self._intern("const", (value.hex(),))

    def inp(self, name: str) -> int:
        if name == "z":
            return self.const(REDSHIFT)
        assert name in INPUT_NAMES, name
        return self._intern("in", (name,))

    def is_const(self, a: int) -> bool:
        return self.nodes[a].op == "const"

    def cval(self, a: int) -> float:
        return float.fromhex(self.nodes[a].args[0])

    def op(self, a: int) -> str:
        return self.nodes[a].op

    def neg(self, a: int) -> int:
        n = self.nodes[a]
        if n.op == "const":
            return self.const(-self.cval(a))
        if n.op == "neg":
            return n.args[0]
        return self._intern("neg", (a,))

    def _split_neg(self, a: int):
        """Return (sign, magnitude node) with sign = -1 when ``a`` is a negation."""
        n = self.nodes[a]
        if n.op == "neg":
            return -1, n.args[0]
        if n.op == "const":
            v = self.cval(a)
            if math.copysign(1.0, v) < 0:
                return -1, self.const(-v)
        return 1, a

    def binary(self, op: str, a: int, b: int) -> int:
        if op in ("add", "sub", "mul", "div"):
            if self.is_const(a) and self.is_const(b):
                x, y = self.cval(a), self.cval(b)
                if op == "add":
                    return self.const(x + y)
                if op == "sub":
                    return self.const(x - y)
                if op == "mul":
                    return self.const(x * y)
                if y != 0.0:
                    return self.const(x / y)
            if op in ("mul", "div"):
                sa, ma = self._split_neg(a)
                sb, mb = self._split_neg(b)
                if op == "mul" and self.is_const(mb) and self.cval(mb) == 1.0:
                    r = ma
                elif op == "mul" and self.is_const(ma) and self.cval(ma) == 1.0:
                    r = mb
                elif op == "div" and self.is_const(mb) and self.cval(mb) == 1.0:
                    r = ma
                else:
                    if op == "mul" and ma > mb:
                        ma, mb = mb, ma
                    r = self._intern(op, (ma, mb))
                return r if sa * sb > 0 else self.neg(r)
            # add / sub: fold signs into the operation
            sa, ma = self._split_neg(a)
            sb, mb = self._split_neg(b)
            if op == "sub":
                sb = -sb
            # now value = sa*ma + sb*mb
            if sa > 0 and sb > 0:
                x, y = sorted((ma, mb))
                return self._intern("add", (x, y))
            if sa > 0 and sb < 0:
                return self._intern("sub", (ma, mb))
            if sa < 0 and sb > 0:
                return self._intern("sub", (mb, ma))
            x, y = sorted((ma, mb))
            return self.neg(self._intern("add", (x, y)))
        if op in ("le", "lt", "ge", "gt", "eq", "ne"):
            # canonical direction: a > b  ==  b < a (exact), a >= b == b <= a
            if op == "gt":
                op, a, b = "lt", b, a
            elif op == "ge":
                op, a, b = "le", b, a
            if op in COMMUTATIVE and a > b:
                a, b = b, a
            return self._intern(op, (a, b), True)
        if op in ("and", "or"):
            av, bv = self._bval(a), self._bval(b)
            if op == "and":
                if av is False or bv is False:
                    return self.bconst(False)
                if av is True:
                    return b
                if bv is True:
                    return a
            else:
                if av is True or bv is True:
                    return self.bconst(True)
                if av is False:
                    return b
                if bv is False:
                    return a
            if a == b:
                return a
            a, b = sorted((a, b))
            return self._intern(op, (a, b), True)
        raise ValueError(op)

    def unary(self, op: str, a: int) -> int:
        n = self.nodes[a]
        if op == "neg":
            return self.neg(a)
        if op == "abs":
            if n.op in ("abs", "exp", "cexp"):
                return a
            if n.op == "neg":
                return self.unary("abs", n.args[0])
            if n.op == "const":
                return self.const(abs(self.cval(a)))
            return self._intern("abs", (a,))
        if op in ("exp", "log", "sqrt"):
            if n.op == "const":
                return self._intern("c" + op, (a,))
            return self._intern(op, (a,))
        if op == "not":
            if n.op == "bconst":
                return self.bconst(not n.args[0])
            if n.op == "not":
                return n.args[0]
            return self._intern("not", (a,), True)
        if op == "b2d":
            return self._intern("b2d", (a,))
        raise ValueError(op)

    def bconst(self, value: bool) -> int:
        return self._intern("bconst", (bool(value),), True)

    def _bval(self, a: int):
        n = self.nodes[a]
        return n.args[0] if n.op == "bconst" else None

    def select(self, c: int, a: int, b: int) -> int:
        if a == b:
            return a
        cv = self._bval(c)
        if cv is not None:
            return a if cv else b
        return self._intern("sel", (c, a, b))

    def bselect(self, c: int, a: int, b: int) -> int:
        """``c ? a : b`` on booleans, written with and/or/not."""
        if a == b:
            return a
        cv = self._bval(c)
        if cv is not None:
            return a if cv else b
        av, bv = self._bval(a), self._bval(b)
        if av is True and bv is False:
            return c
        if av is False and bv is True:
            return self.unary("not", c)
        if av is False:
            return self.binary("and", self.unary("not", c), b)
        if bv is False:
            return self.binary("and", c, a)
        if av is True:
            return self.binary("or", c, b)
        if bv is True:
            return self.binary("or", self.unary("not", c), a)
        return self.binary("or", self.binary("and", c, a),
                           self.binary("and", self.unary("not", c), b))

    # ---------------------------------------------------------------- analysis
    def live_from(self, roots) -> list:
        """Node ids reachable from ``roots`` in topological (creation) order."""
        seen = set()
        stack = list(roots)
        while stack:
            x = stack.pop()
            if x in seen:
                continue
            seen.add(x)
            n = self.nodes[x]
            if n.op not in ("const", "in", "bconst"):
                stack.extend(n.args)
        return sorted(seen)

    def count(self, roots) -> dict:
        out: dict = {}
        for x in self.live_from(roots):
            op = self.nodes[x].op
            out[op] = out.get(op, 0) + 1
        return out

    def weighted(self, counts: dict) -> int:
        return sum(OP_WEIGHT.get(k, 0) * v for k, v in counts.items())

    def rhs_roots(self):
        return [self.outputs[("rhs", i)] for i in range(15)]

    def jac_roots(self):
        return [self.outputs[("jac", r, c)] for r in range(15) for c in range(15)]


def evaluate(dag: Dag, inputs: dict, roots, exp=math.exp, log=math.log, sqrt=math.sqrt):
    """Reference-order evaluation of ``roots`` with Python floats (binary64 RN).

    Used only by the generator's self-checks; branches of ``sel`` are evaluated
    eagerly, which cannot change a selected value.
    """
    vals = {}
    for x in dag.live_from(roots):
        n = dag.nodes[x]
        op, a = n.op, n.args
        if op == "const":
            v = float.fromhex(a[0])
        elif op == "in":
            v = inputs[a[0]]
        elif op == "add":
            v = vals[a[0]] + vals[a[1]]
        elif op == "sub":
            v = vals[a[0]] - vals[a[1]]
        elif op == "mul":
            v = vals[a[0]] * vals[a[1]]
        elif op == "div":
            d = vals[a[1]]
            v = vals[a[0]] / d if d != 0.0 else math.copysign(math.inf, vals[a[0]]) * math.copysign(1.0, d)
        elif op == "neg":
            v = -vals[a[0]]
        elif op == "abs":
            v = abs(vals[a[0]])
        elif op in ("exp", "cexp"):
            try:
                v = exp(vals[a[0]])
            except OverflowError:
                v = math.inf
        elif op in ("log", "clog"):
            u = vals[a[0]]
            v = log(u) if u > 0 else (-math.inf if u == 0 else math.nan)
        elif op in ("sqrt", "csqrt"):
            u = vals[a[0]]
            v = sqrt(u) if u >= 0 else math.nan
        elif op == "le":
            v = vals[a[0]] <= vals[a[1]]
        elif op == "lt":
            v = vals[a[0]] < vals[a[1]]
        elif op == "eq":
            v = vals[a[0]] == vals[a[1]]
        elif op == "ne":
            v = vals[a[0]] != vals[a[1]]
        elif op == "and":
            v = bool(vals[a[0]]) and bool(vals[a[1]])
        elif op == "or":
            v = bool(vals[a[0]]) or bool(vals[a[1]])
        elif op == "not":
            v = not vals[a[0]]
        elif op == "bconst":
            v = a[0]
        elif op == "b2d":
            v = 1.0 if vals[a[0]] else 0.0
        elif op == "sel":
            v = vals[a[1]] if vals[a[0]] else vals[a[2]]
        else:
            raise ValueError(op)
        vals[x] = v
    return [vals[r] for r in roots]
