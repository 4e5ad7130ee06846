"""Text storage of the network DAG (``network.ir``), the committed form of the network.

Format (one record per line, ``#`` starts a comment):

* ``n <id> <op> <args...>``  a node; args are node ids, except ``const`` (a C99 hex
  float literal), ``bconst`` (0/1) and ``in`` (an input name: X0..X13, T);
* ``o rhs <i> <id>``         RHS output i (0..13 species, 14 energy);
* ``o jac <r> <c> <id>``     Jacobian output (row r, column c, both 0-based);
* ``s <group> <op> <count>`` source-level (pre-CSE) operation counts of the
  reference's generated code, used for the algorithmic FLOP count.

Node ids are dense and topologically ordered.  Only nodes reachable from an output
are stored.
"""
from __future__ import annotations

import hashlib
import os

from .network_dag import Dag, Node

DEFAULT_PATH = os.path.join(os.path.dirname(__file__), "network.ir")


def save(dag: Dag, path: str = DEFAULT_PATH, header: str = "") -> str:
    roots = dag.rhs_roots() + dag.jac_roots()
    live = dag.live_from(roots)
    remap = {old: new for new, old in enumerate(live)}
    lines = []
    for line in header.strip().splitlines():
        lines.append("# " + line if line else "#")
    for old in live:
        n = dag.nodes[old]
        if n.op == "const":
            args = [n.args[0]]
        elif n.op == "bconst":
            args = ["1" if n.args[0] else "0"]
        elif n.op == "in":
            args = [n.args[0]]
        else:
            args = [str(remap[a]) for a in n.args]
        lines.append(" ".join(["n", str(remap[old]), n.op] + args))
    for i in range(15):
        lines.append(f"o rhs {i} {remap[dag.outputs[('rhs', i)]]}")
    for r in range(15):
        for c in range(15):
            lines.append(f"o jac {r} {c} {remap[dag.outputs[('jac', r, c)]]}")
    for group in sorted(dag.source_counts):
        for op, cnt in sorted(dag.source_counts[group].items()):
            lines.append(f"s {group} {op} {cnt}")
    text = "\n".join(lines) + "\n"
    with open(path, "w") as f:
        f.write(text)
    return hashlib.sha256(text.encode()).hexdigest()


def load(path: str = DEFAULT_PATH) -> Dag:
    dag = Dag()
    with open(path) as f:
        for raw in f:
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            parts = line.split()
            if parts[0] == "n":
                nid, op = int(parts[1]), parts[2]
                assert nid == len(dag.nodes), "node ids must be dense"
                if op == "const":
                    args = (parts[3],)
                elif op == "bconst":
                    args = (parts[3] == "1",)
                elif op == "in":
                    args = (parts[3],)
                else:
                    args = tuple(int(a) for a in parts[3:])
                    assert all(a < nid for a in args), "nodes must be topological"
                is_bool = op in ("le", "lt", "ge", "gt", "eq", "ne", "and", "or", "not", "bconst")
                dag.nodes.append(Node(op, args, is_bool))
                dag.index[(op, args)] = nid
            elif parts[0] == "o":
                if parts[1] == "rhs":
                    dag.outputs[("rhs", int(parts[2]))] = int(parts[3])
                else:
                    dag.outputs[("jac", int(parts[2]), int(parts[3]))] = int(parts[4])
            elif parts[0] == "s":
                dag.source_counts.setdefault(parts[1], {})[parts[2]] = int(parts[3])
            else:
                raise ValueError(f"bad IR line: {raw!r}")
    assert len([k for k in dag.outputs if k[0] == "rhs"]) == 15
    assert len([k for k in dag.outputs if k[0] == "jac"]) == 225
    return dag


def digest(path: str = DEFAULT_PATH) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()
