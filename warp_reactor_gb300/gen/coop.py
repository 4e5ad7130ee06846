"""Vector programs of the network for the cooperative (lanes-per-cell) advance kernel.

The cooperative kernel evaluates one cell's network with ``G`` lanes (``G`` = 8,
16 or 32 lanes per cell, ``32/G`` cells per warp).  The values of the evaluation
live in the cell's shared-memory slot array ``V``; the work is a *program*: a
sequence of steps, each executed by every lane of the warp, in which lane ``g``
computes one node of the DAG from operands gathered out of ``V`` and stores it
back into ``V``.  Between steps the warp
synchronises, so a step may use any value produced by an earlier step.

Step format (per lane, three 64-bit words; every address is the byte offset of a
slot in the cell's own slot array, so the device adds it to one base):

* main word: four 16-bit fields X | Y | Z | D.  An FMA step computes
  ``V[D] = fma(V[X], V[Y] ^ L, V[Z])``; exp, log and sqrt take ``V[Y] ^ L`` and
  division ``V[X] / (V[Y] ^ L)`` (operands swapped by a flag).  The low three bits
  of a field are free (slots are 8 bytes) and hold flags: the step's class in D,
  "the step has integer nodes" and "they include comparisons or sign operations"
  in Z (both uniform over the step), and the sign modifiers of exp/log/sqrt/div
  arguments in X and Y;
* integer word: four 16-bit fields A | B | C | D2, one integer node
  ``V[D2] = A != 0 ? B : C`` (or a comparison A <= B, A < B, or a sign operation
  on A; the op in the low bits of D2).  Every step may carry up to ``G`` integer
  nodes beside its main node, so comparisons, selects and boolean logic ride
  along with the floating-point work instead of taking steps of their own.
  Boolean logic and copies are selects over the boolean constants:
  a and b = a ? b : 0, a or b = a ? 1 : b, not a = a ? 0 : 1;
* literal word L: the lane's constant operand, XOR-ed into ``V[Y]`` (``Y`` then
  names a slot holding +0.0, so the operand is the constant); 0 otherwise.

Constants therefore never need a table of their own: a network coefficient is the
literal of the lane that uses it, and the few constants that integer nodes and the
outputs read (booleans, the neutral operands 1, -1 and -0, comparison limits) sit
in reserved slots of every cell's array, written once per launch.

Operand modifiers: ``neg`` and ``abs`` nodes of the DAG are never computed.  On an
exp/log/sqrt/div argument they are flags; an FMA or integer node that reads a
negated or absolute value reads it from an integer sign node (``sneg``/``sabs``,
a sign-bit operation, exact) that the generator inserts; on a constant they are
folded into the constant.

Arithmetic: every ``add``, ``sub`` and ``mul`` is one fused multiply-add with
exact neutral operands, so one FP64 instruction class serves all three and lanes
of a step may mix them.  Each is the same correctly rounded binary64 result as
the separate operation:

* ``a * b  == fma(a, b, -0.0)`` (adding -0 never changes a product, and keeps the
  sign of a zero product); ``a * K == fma(a, K, -0.0)``;
* ``a + b  == fma(a, 1.0, b)``, ``a + K == fma(1.0, K, a)`` (the product is
  exact, then one rounding of the sum; IEEE addition commutes);
* ``a - b  == fma(b, -1.0, a)`` (IEEE defines a - b as a + (-b), and b * -1 is
  exactly -b), ``a - K == fma(1.0, -K, a)``, ``K - b == fma(b, -1.0, K)``.

Comparisons are done on the bit patterns (exact IEEE ordering: NaN unordered,
-0 == +0), booleans are stored as the integers 0/1, selects copy bit patterns.

Two programs are generated per ``G``:

* ``jrhs``: inputs ``y[0..14]`` (the ROS2S state: 14 number densities and the
  internal energy); prologue ``burn_state_from_y`` (reproducer.cpp:7029-7038):
  ``X = max(y, 1e-100)`` and ``T = eos_re(X, e)`` (reproducer.cpp:284-314);
  then the fused analytic Jacobian + RHS of ``network.ir``.  The Jacobian's 225
  entries and the RHS are kept values; after the program the kernel gathers
  ``E = -J`` into the matrix slots through the program's Jacobian table (one
  operand per entry ``r*15 + c``, the negation as a modifier);
* ``rhs``: the same prologue and the RHS only.

Slot map of a cell: ``[0, 225)`` the iteration matrix, ``[225, 240)`` the
inputs, ``[240, 240 + R)`` the reserved constants, then scratch; the last slot is
a write sink for idle lanes.  The Jacobian
program runs before the matrix is formed, so it uses the matrix slots as scratch
too and keeps its results above them; the RHS program runs while the matrix holds
the LU factors and never writes it.  Slots are allocated by a linear scan over
the schedule, so the slot count is the largest live set, which sets the shared
memory per cell and hence the cells (warps) per SM.  At 16 lanes per cell (one
cell per half warp) they are allocated bank by bank instead (``allocate_banked``),
so that a step's loads and stores spread over the 16 bank pairs, within the slot
count that keeps the block's warps.

Scheduling is list scheduling by critical path (longest weighted path to an
output) with one class per step; above a live-set limit, nodes whose operands die
with them go first; integer nodes then move as late as their users allow.
Long chains of boolean logic are rebalanced first (``rebalance_boolean_chains``).
Every schedule of the DAG gives the same bits: each node is the same operation on
the same operands wherever and whenever it is computed.
"""
from __future__ import annotations

import collections
import os
import random
import struct

from . import ir_io

# main classes
C_NONE, C_FMA, C_EXP, C_LOG, C_SQRT, C_DIV = 0, 1, 2, 3, 4, 5
# integer ops: every copy / and / or / not / select is one select A ? B : C (with
# the boolean constants 0 and 1 as operands); comparisons A <= B, A < B; a sign
# operation on A (flip the sign bit, or clear it)
I_SEL, I_LE, I_LT, I_SGN = 0, 1, 2, 3

FMA_OPS = ("add", "sub", "mul")
MAIN_CLASS = {"add": C_FMA, "sub": C_FMA, "mul": C_FMA, "exp": C_EXP, "cexp": C_EXP, "log": C_LOG,
              "clog": C_LOG, "sqrt": C_SQRT, "csqrt": C_SQRT, "div": C_DIV}
INT_OP = {"le": I_LE, "lt": I_LT, "and": I_SEL, "or": I_SEL, "not": I_SEL, "sel": I_SEL, "sneg": I_SGN,
          "sabs": I_SGN}
# FP64 issue slots of one step of each class (measured call throughput of CUDA's
# exp/log/sqrt on GB300; division runs on the integer pipe)
STEP_COST = {C_FMA: 1.0, C_EXP: 19.0, C_LOG: 29.0, C_SQRT: 9.0, C_DIV: 0.5}
# latency weights for the critical-path priority
LATENCY = {C_FMA: 1.0, C_EXP: 3.0, C_LOG: 3.0, C_SQRT: 2.0, C_DIV: 2.0, "int": 1.0}

E_SLOTS = 225
Y_BASE = 225
RES_BASE = 240
SLOT_BITS = 12
MAX_SLOTS = 1 << SLOT_BITS
# output operands (the RHS and Jacobian tables): slot | negate | absolute value
OPF_NEG = 1 << 13
OPF_ABS = 1 << 14
# flags in the low bits of the 16-bit address fields (slots are 8 bytes)
FL_NEG, FL_ABS, FL_SWAP = 1, 2, 4        # X, Y: argument modifiers; Y: divide V[Y] ^ L by V[X]
FL_INT, FL_SPECIAL = 1, 2                # Z: the step has integer nodes / comparisons or sign ops
FL_SABS = 4                              # D2 of I_SGN: clear the sign bit (else flip it)
# steps are executed in groups of four, and the tables carry four idle steps more
# so that the device may load four steps ahead without a bound check
STEP_ALIGN = 4
PREFETCH_PAD = 4
SIGN = 1 << 63
ABS = SIGN - 1
# leaves of a program: inputs, constants, and transcendentals of constants
# ("dconst": evaluated once per launch on the device, with the kernel's own
# exp/log/sqrt, into reserved slots)
LEAF = ("in", "const", "dconst")
TRANSCENDENTAL = {"exp": C_EXP, "cexp": C_EXP, "log": C_LOG, "clog": C_LOG, "sqrt": C_SQRT, "csqrt": C_SQRT}

FLOOR = 1.0e-100  # reproducer.cpp:231
# species masses, reproducer.cpp:233-248 (the literals of wr_physics.cuh)
MASS = (9.10938188e-28, 1.67262158e-24, 1.67353251819e-24, 1.67444345638e-24, 3.34512158e-24,
        3.34603251819e-24, 3.34615409819e-24, 3.34694345638e-24, 3.34706503638e-24, 5.01865409819e-24,
        5.01956503638e-24, 6.69024316e-24, 6.69115409819e-24, 6.69206503638e-24)
K_MP = 1.67262192595e-24
K_GAS = 6.02214076e+23 * 1.3806490000000002e-16


def inv_gm1(n: int) -> float:
    return 1.0 / ((1.4 if n in (6, 8, 9, 10) else 5.0 / 3.0) - 1.0)


def dbits(v: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", v))[0]


class Program:
    """A DAG in program form: nodes (op, args), leaves 'in'/'const'."""

    def __init__(self):
        self.nodes = []      # (op, args); const: ('const', (bits,)); in: ('in', (k,))
        self.cmemo = {}

    def add(self, op, *args):
        self.nodes.append((op, tuple(args)))
        return len(self.nodes) - 1

    def const_bits(self, bits: int):
        if bits not in self.cmemo:
            self.cmemo[bits] = self.add("const", bits)
        return self.cmemo[bits]

    def const(self, v: float):
        return self.const_bits(dbits(v))


def build(dag, kind: str) -> tuple:
    """The program of ``kind`` ('jrhs' or 'rhs') and its outputs:
    ``jac`` {(r, c): node} (jrhs only) and ``rhs`` [node] * 15."""
    P = Program()
    Y = [P.add("in", k) for k in range(15)]
    floor = P.const(FLOOR)
    # burn_state_from_y: X = smax(y, floor) = (y < floor) ? floor : y
    X = [P.add("sel", P.add("lt", Y[k], floor), floor, Y[k]) for k in range(14)]
    # eos_re (eos_sums + T): the sums start from 0.0, and 0.0 + v == v for the
    # products/terms here (positive: X >= 1e-100, or NaN), so the first add is dropped
    rhotot = P.add("mul", X[0], P.const(MASS[0]))
    for n in range(1, 14):
        rhotot = P.add("add", rhotot, P.add("mul", X[n], P.const(MASS[n])))
    sa = X[0]
    for n in range(1, 14):
        sa = P.add("add", sa, X[n])
    sg = None
    for n in range(14):
        term = P.add("mul", P.add("div", P.add("mul", X[n], P.const(K_MP)), rhotot), P.const(inv_gm1(n)))
        sg = term if sg is None else P.add("add", sg, term)
    sa = P.add("mul", sa, P.add("div", P.const(K_MP), rhotot))
    sg = P.add("div", sg, sa)
    T = P.add("div", Y[14], P.add("mul", P.add("mul", sg, P.const(K_GAS)), sa))
    # the network with X, T substituted
    roots = dag.rhs_roots() + (dag.jac_roots() if kind == "jrhs" else [])
    live = dag.live_from(roots)
    m = {}
    for x in live:
        n = dag.nodes[x]
        if n.op == "in":
            m[x] = T if n.args[0] == "T" else X[int(n.args[0][1:])]
        elif n.op == "const":
            m[x] = P.const(float.fromhex(n.args[0]))
        elif n.op == "bconst":
            m[x] = P.const_bits(1 if n.args[0] else 0)
        else:
            m[x] = P.add(n.op, *[m[a] for a in n.args])
    out = {"rhs": [m[dag.outputs[("rhs", i)]] for i in range(15)]}
    if kind == "jrhs":
        out["jac"] = {(r, c): m[dag.outputs[("jac", r, c)]] for r in range(15) for c in range(15)}
    rebalance_boolean_chains(P)
    return P, out


BOOL_OPS = ("and", "or", "not")


def rebalance_boolean_chains(P: Program, min_depth: int = 12):
    """Shorten long chains of boolean logic.

    The network holds conditions folded over many terms, c_k+1 = or(a_k,
    and(c_k, not(b_k))), ~150 levels deep: evaluated as written they need one
    step each at the end of the RHS program.  Along such a chain (each link
    the only user of the one below) every link is a map of the chain value c in
    {0, 1}: and(c, s) -> (0, s), or(c, s) -> (s, 1), not(c) -> (1, 0), written
    as the pair (value at c = 0, value at c = 1).  Maps compose exactly,
    (g o f)(i) = f(i) ? g(1) : g(0), so a balanced tree of compositions gives the
    whole chain's map in log2(length) levels of selects, and the top node
    becomes sel(c_0, map(1), map(0)).  Booleans are the integers 0 and 1, so
    the value of every node is unchanged."""
    zero, one = P.const_bits(0), P.const_bits(1)
    memo = {}

    def sel(c, a, b):
        if c == one:
            return a
        if c == zero or a == b:
            return b
        if a == one and b == zero:
            return c
        key = ("sel", c, a, b)
        if key not in memo:
            memo[key] = P.add("sel", c, a, b)
        return memo[key]

    def compose(g, f):  # g after f
        return sel(f[0], g[1], g[0]), sel(f[1], g[1], g[0])

    while True:
        users = collections.defaultdict(list)
        depth = {}
        for i, (op, a) in enumerate(P.nodes):
            if op in ("in", "const"):
                continue
            for y in a:
                users[y].append(i)
            if op in BOOL_OPS:
                depth[i] = 1 + max((depth.get(y, 0) for y in a), default=0)
        if not depth:
            return
        top = max(depth, key=lambda x: (depth[x], -x))
        if depth[top] < min_depth:
            return
        # the chain below top: follow the deepest boolean operand while it has
        # no other user
        links = []  # (node, chain operand) from the top down
        x = top
        while P.nodes[x][0] in BOOL_OPS:
            op, a = P.nodes[x]
            below = max(a, key=lambda y: depth.get(y, 0))
            links.append((x, below))
            if depth.get(below, 0) == 0 or len(users[below]) != 1 or P.nodes[below][0] not in BOOL_OPS:
                break
            x = below
        if len(links) < min_depth:
            return
        maps = []  # bottom-up link maps
        for x, below in reversed(links):
            op, a = P.nodes[x]
            if op == "not":
                maps.append((one, zero))
            else:
                other = a[1] if a[0] == below else a[0]
                maps.append((zero, other) if op == "and" else (other, one))
        while len(maps) > 1:
            nxt = [compose(maps[i + 1], maps[i]) for i in range(0, len(maps) - 1, 2)]
            if len(maps) % 2:
                nxt.append(maps[-1])
            maps = nxt
        m0, m1 = maps[0]
        c0 = links[-1][1]
        P.nodes[top] = ("sel", (c0, m1, m0))


def resolve(P: Program, x: int):
    """(base node, neg, abs) of x with neg/abs nodes folded into modifiers."""
    chain = []
    while P.nodes[x][0] in ("neg", "abs"):
        chain.append(P.nodes[x][0])
        x = P.nodes[x][1][0]
    neg = ab = False
    for op in reversed(chain):  # innermost first
        if op == "neg":
            neg = not neg
        else:
            ab, neg = True, False
    return x, neg, ab


def lower(P: Program) -> None:
    """Take operand modifiers off the operands of FMA and integer nodes, whose step
    format reads plain slots: a negated or absolute operand becomes an integer
    sign node (``sabs`` then ``sneg``, shared by every reader of the same value),
    and a modified constant becomes the constant with that sign.  Arguments of
    exp/log/sqrt/div keep their modifiers (flags of their step format).

    An exp, log or sqrt of a constant becomes a ``dconst`` leaf (class, argument
    bits): the kernel evaluates it once per launch with its own math functions,
    so every program run reads the same bits it would have computed."""
    memo = {}
    for x in range(len(P.nodes)):
        op, a = P.nodes[x]
        if op in TRANSCENDENTAL:
            b, neg, ab = resolve(P, a[0])
            if P.nodes[b][0] == "const":
                bits = P.nodes[b][1][0]
                bits = (bits & ABS) if ab else bits
                P.nodes[x] = ("dconst", (TRANSCENDENTAL[op], bits ^ SIGN if neg else bits))

    def plain(y):
        b, neg, ab = resolve(P, y)
        if not (neg or ab):
            return b
        if P.nodes[b][0] == "const":
            bits = P.nodes[b][1][0]
            bits = (bits & ABS) if ab else bits
            return P.const_bits(bits ^ SIGN if neg else bits)
        key = (b, neg, ab)
        if key not in memo:
            t = P.add("sabs", b) if ab else b
            memo[key] = P.add("sneg", t) if neg else t
        return memo[key]

    for x in range(len(P.nodes)):
        op, a = P.nodes[x]
        if op in FMA_OPS or op in INT_OP:
            P.nodes[x] = (op, tuple(plain(y) for y in a))


def live_nodes(P: Program, roots, leaves=False) -> list:
    """The computed nodes the roots depend on (neg/abs folded), sorted; with
    ``leaves``, the leaves they read too."""
    leaf = LEAF
    seen, stack = set(), [resolve(P, r)[0] for r in roots]
    while stack:
        x = stack.pop()
        if x in seen:
            continue
        seen.add(x)
        op, a = P.nodes[x]
        if op in leaf:
            continue
        for y in a:
            stack.append(resolve(P, y)[0])
    return sorted(x for x in seen if leaves or P.nodes[x][0] not in leaf)


def roots_of(out: dict) -> list:
    return list(out["rhs"]) + ([x for _, x in sorted(out["jac"].items())] if "jac" in out else [])


def device_constants(P: Program, out: dict) -> set:
    """The (class, argument bits) of the program's transcendentals of constants."""
    return {P.nodes[x][1] for x in live_nodes(P, roots_of(out), leaves=True) if P.nodes[x][0] == "dconst"}


def reserved_constants(P: Program, out: dict) -> set:
    """Constants the program reads from reserved slots: the operands of integer
    nodes, the minuend of K - b, and constant outputs."""
    res = set()
    for x in live_nodes(P, roots_of(out)):
        op, a = P.nodes[x]
        if op in INT_OP or op == "sub":
            for y in (a if op in INT_OP else a[:1]):
                b = resolve(P, y)[0]
                if P.nodes[b][0] == "const":
                    res.add(P.nodes[b][1][0])
    for r in roots_of(out):
        b = resolve(P, r)[0]
        if P.nodes[b][0] == "const":
            res.add(P.nodes[b][1][0])
    return res


class Schedule:
    def __init__(self, G, steps, slot, nv, outputs, consts):
        self.G = G
        self.steps = steps        # [(cls, [main node], [int node])]
        self.slot = slot          # node -> slot
        self.nv = nv
        self.outputs = outputs
        self.consts = consts


def list_schedule(comp, args, users, kind, prio, G, limit=None, hold=None):
    """Steps of width G: each step takes up to G ready nodes of one main class
    (highest priority first; a full step is preferred) and up to G ready integer
    nodes.  ``args``/``users`` give the dependences in the direction scheduled.

    ``hold``: a partial exp/log/sqrt step costs as many FP64 issue slots as a full
    one, so while an FMA or division step can be filled instead, a transcendental
    class is taken only if its most critical ready node leads theirs by more than
    ``hold`` (a number, or one per class; None: no such rule).

    ``limit``: once that many computed values are live (computed, with users not
    yet scheduled), ready nodes are taken by their effect on the live set first
    (a node whose operands die with it before one that only adds a value), then
    by priority: the cell's shared memory is set by the largest live set."""
    pend = {x: len(set(args[x])) for x in comp}
    remaining = {x: len(set(users[x])) for x in comp}
    ready = collections.defaultdict(list)
    for x in comp:
        if pend[x] == 0:
            ready[kind(x)].append(x)
    steps = []
    left = len(comp)
    live = 0
    mains = (C_FMA, C_EXP, C_LOG, C_SQRT, C_DIV)

    def key(x):
        if limit is not None and live >= limit:
            freed = sum(1 for a in set(args[x]) if remaining[a] == 1)
            return ((1 if users[x] else 0) - freed, -prio[x])
        return (0, -prio[x])

    def top(c):
        return max(prio[x] for x in ready[c])

    while left:
        rl = sorted(ready["int"], key=key)
        riders, ready["int"] = rl[:G], rl[G:]
        cand = [c for c in mains if ready[c]]
        cls, take = C_NONE, []
        if cand:
            full = [c for c in cand if len(ready[c]) >= G]
            pool = full if full else cand
            cheap = [c for c in cand if c in (C_FMA, C_DIV)]
            if hold is not None and not full and cheap:
                lead = max(top(c) for c in cheap)
                hc = hold if isinstance(hold, dict) else {c: hold for c in mains}
                pool = cheap + [c for c in cand if c not in cheap and top(c) > lead + hc.get(c, 0.0)]
            cls = max(pool, key=lambda c: (top(c), len(ready[c])))
            rl = sorted(ready[cls], key=key)
            take, ready[cls] = rl[:G], rl[G:]
        steps.append((cls, take, riders))
        left -= len(take) + len(riders)
        for x in take + riders:
            live += 1 if users[x] else 0
            for a in set(args[x]):
                remaining[a] -= 1
                live -= 1 if remaining[a] == 0 else 0
            for u in users[x]:
                pend[u] -= 1
                if pend[u] == 0:
                    ready[kind(u)].append(u)
    return steps


def sink_riders(steps, users, kind, G):
    """Move every integer node with users to the latest step before its first
    user that has a free integer lane (integer nodes cost no FP64 issue slot, so
    computing them late only shortens their values' lives); steps left empty are
    dropped."""
    done = {}
    for s, (_, take, riders) in enumerate(steps):
        for x in take + riders:
            done[x] = s
    lanes = [list(r) for _, _, r in steps]
    for x in sorted((x for x in done if kind(x) == "int" and users[x]), key=lambda x: -done[x]):
        first_use = min(done[u] for u in users[x])
        for s in range(first_use - 1, done[x], -1):
            if len(lanes[s]) < G:
                lanes[done[x]].remove(x)
                lanes[s].append(x)
                done[x] = s
                break
    return [(cls, take, lanes[s]) for s, (cls, take, _) in enumerate(steps) if take or lanes[s]]


def schedule(P: Program, out: dict, G: int, jac: bool, limit=None, first_scratch=RES_BASE, tune=None,
             banked=None):
    """List-schedule the program into steps of width G and allocate slots.

    ``jac``: the program computes the Jacobian too.  Its 225 entries are kept
    values like the RHS (no matrix slot is reserved while the program runs, so
    the iteration matrix's slots serve as scratch); after the program the kernel
    gathers E = -J into the matrix slots from the ``jac`` output table.  Kept
    values therefore live above the matrix slots.  The RHS-only program runs
    while the matrix holds LU factors, so it never writes the matrix slots.
    ``first_scratch``: the first slot above the reserved constants.  ``tune``:
    (latency weight of exp/log/sqrt, ``hold`` of the list scheduler, seed of a
    random perturbation of the priorities (0: none)[, its amplitude, 1e-3 by
    default]) -- the schedule is a heuristic, and these pick among equally valid
    ones.  ``banked``: (reserved slot map, slot cap) to allocate slots with
    ``allocate_banked`` (G = 16), falling back to the linear scan when it finds
    no room below the cap."""
    leaf = LEAF
    jac_roots = [x for _, x in sorted(out["jac"].items())] if jac else []
    roots = list(out["rhs"]) + jac_roots
    comp = live_nodes(P, roots)
    args = {x: [resolve(P, a)[0] for a in P.nodes[x][1]] for x in comp}
    cargs = {x: sorted({a for a in args[x] if P.nodes[a][0] not in leaf}) for x in comp}
    users = collections.defaultdict(list)
    for x in comp:
        for a in cargs[x]:
            users[a].append(x)

    def kind(x):
        return MAIN_CLASS.get(P.nodes[x][0], "int")

    # topological order (node indices are not one: rewrites add operands late)
    pend = {x: len(cargs[x]) for x in comp}
    order = [x for x in comp if pend[x] == 0]
    for x in order:
        for u in users[x]:
            pend[u] -= 1
            if pend[u] == 0:
                order.append(u)
    assert len(order) == len(comp), "the program has a cycle"
    lat_t, hold, seed, amp = (tuple(tune) + (1e-3,))[:4] if tune else (LATENCY[C_EXP], None, 0, 0.0)
    lat = dict(LATENCY)
    lat.update({C_EXP: lat_t, C_LOG: lat_t, C_SQRT: max(1.0, lat_t - 1.0)})
    rng = random.Random(seed)
    prio = {}
    for x in reversed(order):
        prio[x] = lat[kind(x)] + max((prio[u] for u in users[x]), default=0.0)
        prio[x] += rng.random() * amp if seed else 0.0
    steps = sink_riders(list_schedule(comp, cargs, users, kind, prio, G, limit, hold), users, kind, G)
    done_at = {}
    for s, (cls, take, riders) in enumerate(steps):
        for x in take + riders:
            done_at[x] = s
    for x in comp:
        assert all(done_at[a] < done_at[x] for a in cargs[x]), "schedule violates a dependence"
    # ---- slot allocation (linear scan; a slot read last in step s is free from
    # s+1).  Two pools: the matrix slots (scratch of the Jacobian program only)
    # and the slots above the inputs; kept values come from the upper pool.
    import heapq
    last = {}
    for s, (cls, take, riders) in enumerate(steps):
        for x in take + riders:
            for a in args[x]:
                if P.nodes[a][0] == "in" or P.nodes[a][0] not in leaf:
                    last[a] = s
    keep = {resolve(P, r)[0] for r in roots}
    inputs = [x for x in range(len(P.nodes)) if P.nodes[x][0] == "in"]
    if banked is not None and G == BANKS:
        got = allocate_banked(P, steps, last, keep, inputs, banked[0], jac, first_scratch, banked[1] - 1)
        if got is not None:
            slot, nv = got
            outputs = {"rhs": [resolve(P, r) for r in out["rhs"]]}
            if jac:
                outputs["jac"] = [resolve(P, x) for x in jac_roots]
            return Schedule(G, steps, slot, nv + 1, outputs, None), args  # + the write sink
    slot = {}
    low = list(range(E_SLOTS)) if jac else []  # min-heaps of free slots
    high = []
    next_slot = first_scratch
    release = collections.defaultdict(list)
    for x in inputs:
        slot[x] = Y_BASE + P.nodes[x][1][0]
        if x in keep:
            continue
        if x in last:
            release[last[x] + 1].append(slot[x])
        else:
            heapq.heappush(high, slot[x])
    nv = next_slot
    for s, (cls, take, riders) in enumerate(steps):
        for sl in release.pop(s, []):
            heapq.heappush(low if sl < E_SLOTS else high, sl)
        for x in take + riders:
            if low and x not in keep:
                sl = heapq.heappop(low)
            elif high:
                sl = heapq.heappop(high)
            else:
                sl = next_slot
                next_slot += 1
            slot[x] = sl
            if x not in keep:
                release[last.get(x, s) + 1].append(sl)
        nv = max(nv, next_slot)
    nv += 1  # write sink of idle lanes
    if nv > MAX_SLOTS:
        raise ValueError(f"program needs {nv} slots (max {MAX_SLOTS})")
    outputs = {"rhs": [resolve(P, r) for r in out["rhs"]]}
    if jac:
        outputs["jac"] = [resolve(P, x) for x in jac_roots]
    return Schedule(G, steps, slot, nv, outputs, None), args


def operand_refs(P: Program, x: int, res: dict) -> dict:
    """The operands the interpreter loads for node x, by field (X, Y, Z of a main
    node; A, B, C of an integer node), as ``encode`` lays them out: ``("n", node)``
    for a computed value, ``("s", slot)`` for a fixed slot (an input, a reserved
    constant, a transcendental of a constant).  A constant that rides as the
    lane's literal loads the +0.0 slot."""
    ZERO, IONE, ONE, MONE, MZERO = (("s", res[b]) for b in (0, 1, dbits(1.0), dbits(-1.0), dbits(-0.0)))

    def const(y):
        return P.nodes[resolve(P, y)[0]][0] == "const"

    def ref(y):
        b = resolve(P, y)[0]
        op, a = P.nodes[b]
        if op == "const":
            return ("s", res[a[0]])
        if op == "dconst":
            return ("s", res[a])
        if op == "in":
            return ("s", Y_BASE + a[0])
        return ("n", b)

    op, a = P.nodes[x]
    if op == "mul":
        if const(a[0]) or const(a[1]):
            return {"X": ref(a[1] if const(a[0]) else a[0]), "Y": ZERO, "Z": MZERO}
        return {"X": ref(a[0]), "Y": ref(a[1]), "Z": MZERO}
    if op == "add":
        if const(a[0]) or const(a[1]):
            return {"X": ONE, "Y": ZERO, "Z": ref(a[1] if const(a[0]) else a[0])}
        return {"X": ref(a[0]), "Y": ONE, "Z": ref(a[1])}
    if op == "sub":
        if const(a[1]):
            return {"X": ONE, "Y": ZERO, "Z": ref(a[0])}
        return {"X": ref(a[1]), "Y": MONE, "Z": ref(a[0])}
    if op == "div":
        if const(a[0]):
            return {"X": ref(a[1]), "Y": ZERO}
        if const(a[1]):
            return {"X": ref(a[0]), "Y": ZERO}
        return {"X": ref(a[0]), "Y": ref(a[1])}
    if op in MAIN_CLASS:  # exp, log, sqrt
        return {"Y": ZERO if const(a[0]) else ref(a[0])}
    if op == "and":
        return {"A": ref(a[0]), "B": ref(a[1]), "C": ZERO}
    if op == "or":
        return {"A": ref(a[0]), "B": IONE, "C": ref(a[1])}
    if op == "not":
        return {"A": ref(a[0]), "B": ZERO, "C": IONE}
    if op == "sel":
        return {"A": ref(a[0]), "B": ref(a[1]), "C": ref(a[2])}
    if op in ("le", "lt"):
        return {"A": ref(a[0]), "B": ref(a[1]), "C": ONE}
    return {"A": ref(a[0]), "B": ONE, "C": ONE}  # sneg, sabs


def _assign(cost) -> list:
    """Minimum-cost assignment of n rows to distinct columns of an n x m cost
    matrix (n <= m; Hungarian method with potentials): the column of each row."""
    n, m = len(cost), len(cost[0])
    INF = float("inf")
    u, v = [0.0] * (n + 1), [0.0] * (m + 1)
    p, way = [0] * (m + 1), [0] * (m + 1)
    for i in range(1, n + 1):
        p[0] = i
        j0 = 0
        minv = [INF] * (m + 1)
        used = [False] * (m + 1)
        while True:
            used[j0] = True
            i0, delta, j1 = p[j0], INF, 0
            for j in range(1, m + 1):
                if not used[j]:
                    cur = cost[i0 - 1][j - 1] - u[i0] - v[j]
                    if cur < minv[j]:
                        minv[j], way[j] = cur, j0
                    if minv[j] < delta:
                        delta, j1 = minv[j], j
            for j in range(m + 1):
                if used[j]:
                    u[p[j]] += delta
                    v[j] -= delta
                else:
                    minv[j] -= delta
            j0 = j1
            if p[j0] == 0:
                break
        while j0:
            j1 = way[j0]
            p[j0] = p[j1]
            j0 = j1
    col = [0] * n
    for j in range(1, m + 1):
        if p[j]:
            col[p[j] - 1] = j - 1
    return col


BANKS = 16  # bank pairs of a 64-bit shared access by one half warp
# allocate_banked: cost per slot of a bank's planned occupancy within BANK_MARGIN
# of its room (chosen with shared_wavefronts: 1 and 2.0 give the fewest)
BANK_MARGIN = 1
BANK_FILL = 2.0


def allocate_banked(P: Program, steps, last, keep, inputs, res, jac: bool, first_scratch: int, cap: int):
    """Slot allocation that spreads every shared access of a half warp (one cell's
    16 lanes) over the 16 bank pairs (slot mod 16).

    Each value's bank is chosen when its step is allocated, by a minimum-cost
    assignment of the step's new values (main nodes, then integer nodes) to banks:
    - a value costs one for every value already placed in that bank that is
      loaded beside it (the same field of a step that reads both) and for every
      fixed slot there (inputs, reserved constants);
    - a second value of the step in one bank costs one (its store replays);
    - the bank's planned occupancy over the value's lifetime (every placed value
      is counted from its step to its last read) may not exceed the bank's slots
      below ``cap``, and costs ``BANK_FILL`` per slot when it comes within
      ``BANK_MARGIN`` of them: a bank that fills early would force conflicts (or
      more slots) later.
    Lifetimes are those of the linear scan: a slot read last in step s is free
    from s + 1, so no step reads a slot that it also writes.  A value takes the
    lowest free slot of its bank (the matrix slots first, for a Jacobian-program
    value that is not kept), else the bank's next slot above ``first_scratch``.
    Returns the slot map and the slot count, or None when a step finds no room."""
    import heapq
    groups, reads = [], collections.defaultdict(list)

    def group(refs, idle):
        fixed = [0] * BANKS
        for r in set(refs) | ({idle} if idle else set()):
            if r[0] == "s":
                fixed[r[1] % BANKS] += 1
            else:
                reads[r[1]].append(len(groups))
        groups.append(fixed)

    ONE = ("s", res[dbits(1.0)])
    for cls, take, riders in steps:
        if cls != C_NONE:
            maps = [operand_refs(P, x, res) for x in take]
            for f in {C_FMA: "XYZ", C_DIV: "XY"}.get(cls, "Y"):
                group([m[f] for m in maps], ONE if len(take) < BANKS else None)
        if riders:
            maps = [operand_refs(P, x, res) for x in riders]
            short = len(riders) < BANKS
            for f, idle in (("A", ("s", res[1])), ("B", ONE), ("C", ONE)):
                group([m[f] for m in maps], idle if short else None)

    S = len(steps)
    end = {x: S + 1 if x in keep else last.get(x, s) for s, (_, take, riders) in enumerate(steps)
           for x in take + riders}
    room = [0] * BANKS  # slots of each bank: matrix (Jacobian program), inputs, scratch
    for sl in [*range(E_SLOTS if jac else 0), *range(Y_BASE, RES_BASE), *range(first_scratch, cap)]:
        room[sl % BANKS] += 1
    occ = [[0] * (S + 2) for _ in range(BANKS)]
    free = {"low": [[] for _ in range(BANKS)], "high": [[] for _ in range(BANKS)]}
    if jac:
        for sl in range(E_SLOTS):
            heapq.heappush(free["low"][sl % BANKS], sl)
    nxt = [first_scratch + ((b - first_scratch) % BANKS) for b in range(BANKS)]
    slot = {}
    release = collections.defaultdict(list)
    for x in inputs:
        slot[x] = sl = Y_BASE + P.nodes[x][1][0]
        e = S + 1 if x in keep else last.get(x, -1)
        for t in range(e + 1):
            occ[sl % BANKS][t] += 1
        if x in keep:
            continue
        if x in last:
            release[last[x] + 1].append(sl)
        else:
            heapq.heappush(free["high"][sl % BANKS], sl)
    top = first_scratch - 1
    for s, (cls, take, riders) in enumerate(steps):
        for sl in release.pop(s, []):
            heapq.heappush(free["low" if sl < E_SLOTS else "high"][sl % BANKS], sl)
        for nodes in (take, riders):
            if not nodes:
                continue
            cost = []
            for x in nodes:
                pools = ("high",) if x in keep else ("low", "high")
                row = []
                for b in range(BANKS):
                    peak = max(occ[b][s:end[x] + 1])
                    if peak + 1 > room[b] or (nxt[b] >= cap and not any(free[p][b] for p in pools)):
                        row.append(1e9)
                        continue
                    fill = max(0, peak + 1 - (room[b] - BANK_MARGIN))
                    row.append(BANK_FILL * fill + sum(groups[g][b] for g in reads[x]))
                cost.append(row + [c + 1.0 for c in row])
            for x, col, row in zip(nodes, _assign(cost), cost):
                if row[col] >= 1e9:
                    return None
                b = col % BANKS
                pools = ("high",) if x in keep else ("low", "high")
                pool = next((p for p in pools if free[p][b]), None)
                if pool is not None:
                    sl = heapq.heappop(free[pool][b])
                else:
                    sl = nxt[b]
                    nxt[b] += BANKS
                    top = max(top, sl)
                slot[x] = sl
                for t in range(s, end[x] + 1):
                    occ[b][t] += 1
                for g in reads[x]:
                    groups[g][b] += 1
                if x not in keep:
                    release[last.get(x, s) + 1].append(sl)
    return slot, max(top + 1, first_scratch)


def encode(P: Program, sch: Schedule, res: dict) -> list:
    """Per-step, per-lane (main, integer, literal) words; ``res`` maps the bits of
    each reserved constant, and the (class, argument bits) of each transcendental
    of a constant, to its slot.  Steps are padded with idle steps (all
    words zero) to a multiple of ``STEP_ALIGN``, then ``PREFETCH_PAD`` more."""
    G = sch.G
    ZERO, IONE, ONE, MONE, MZERO = (res[b] for b in (0, 1, dbits(1.0), dbits(-1.0), dbits(-0.0)))
    sink = sch.nv - 1

    def const(x):
        return P.nodes[resolve(P, x)[0]][0] == "const"

    def cbits(x):  # a constant operand with its modifiers applied
        b, neg, ab = resolve(P, x)
        bits = P.nodes[b][1][0]
        bits = (bits & ABS) if ab else bits
        return bits ^ SIGN if neg else bits

    def slot_of(b):
        op = P.nodes[b][0]
        return res[P.nodes[b][1][0]] if op == "const" else res[P.nodes[b][1]] if op == "dconst" else sch.slot[b]

    def plain(x):  # slot of an operand without modifiers (constants: reserved)
        b, neg, ab = resolve(P, x)
        assert not (neg or ab), "operand modifier left on an FMA or integer node"
        return slot_of(b)

    def arg(x):  # slot and modifier flags of an exp/log/sqrt/div argument
        b, neg, ab = resolve(P, x)
        return slot_of(b), (FL_NEG if neg else 0) | (FL_ABS if ab else 0)

    words = []
    for cls, take, riders in sch.steps:
        special = any(P.nodes[x][0] in ("le", "lt", "sneg", "sabs") for x in riders)
        zfl = (FL_INT if riders else 0) | (FL_SPECIAL if special else 0)
        lanes = []
        for g in range(G):
            xf = yf = 0
            L = 0
            X = Y = Z = ONE
            dst = sink
            if g < len(take):
                x = take[g]
                op, a = P.nodes[x]
                if op in FMA_OPS:
                    assert not (const(a[0]) and const(a[1])), "FMA node of two constants"
                if op == "mul":
                    if const(a[0]) or const(a[1]):
                        v, k = (a[1], a[0]) if const(a[0]) else (a[0], a[1])
                        X, Y, Z, L = plain(v), ZERO, MZERO, cbits(k)
                    else:
                        X, Y, Z = plain(a[0]), plain(a[1]), MZERO
                elif op == "add":
                    if const(a[0]) or const(a[1]):
                        v, k = (a[1], a[0]) if const(a[0]) else (a[0], a[1])
                        X, Y, Z, L = ONE, ZERO, plain(v), cbits(k)
                    else:
                        X, Y, Z = plain(a[0]), ONE, plain(a[1])
                elif op == "sub":
                    if const(a[1]):  # a - K = fma(1, -K, a)
                        X, Y, Z, L = ONE, ZERO, plain(a[0]), cbits(a[1]) ^ SIGN
                    else:  # a - b = fma(b, -1, a); K - b reads K from its reserved slot
                        X, Y, Z = plain(a[1]), MONE, plain(a[0])
                elif op == "div":
                    num, den = a
                    if const(num):  # K / b: V[Y] ^ L = K, divided by V[X] = b
                        (X, xf), Y, L, yf = arg(den), ZERO, cbits(num), FL_SWAP
                    elif const(den):
                        (X, xf), Y, L = arg(num), ZERO, cbits(den)
                    else:
                        (X, xf), (Y, yf) = arg(num), arg(den)
                else:  # exp, log, sqrt (and their constant-argument forms)
                    if const(a[0]):
                        Y, L = ZERO, cbits(a[0])
                    else:
                        Y, yf = arg(a[0])
                dst = sch.slot[x]
            main = ((X << 3) | xf) | (((Y << 3) | yf) << 16) | (((Z << 3) | zfl) << 32) | (((dst << 3) | cls) << 48)
            A, B, C, iop, idst = IONE, ONE, ONE, I_SEL, sink
            if g < len(riders):
                x = riders[g]
                op, a = P.nodes[x]
                iop = INT_OP[op]
                if op == "and":
                    A, B, C = plain(a[0]), plain(a[1]), ZERO
                elif op == "or":
                    A, B, C = plain(a[0]), IONE, plain(a[1])
                elif op == "not":
                    A, B, C = plain(a[0]), ZERO, IONE
                elif op == "sel":
                    A, B, C = plain(a[0]), plain(a[1]), plain(a[2])
                elif op in ("le", "lt"):
                    A, B = plain(a[0]), plain(a[1])
                else:  # sneg, sabs
                    A = plain(a[0])
                    iop |= FL_SABS if op == "sabs" else 0
                idst = sch.slot[x]
            rider = (A << 3) | ((B << 3) << 16) | ((C << 3) << 32) | (((idst << 3) | iop) << 48)
            lanes.append((main, rider, L))
        words.append(lanes)
    idle = [(0, 0, 0)] * G
    while len(words) % STEP_ALIGN:
        words.append(idle)
    return words + [idle] * PREFETCH_PAD


# live-set limit of the list scheduler per G (chosen offline: the smallest slot
# count among limits that do not add FP64 issue slots)
SCHED_LIMIT = {8: 400, 16: 650, 32: None}
# scheduler tuning per G and program: (schedule()'s ``tune``, live-set limit),
# chosen offline by a seeded random search for the fewest FP64 issue slots of the
# program whose slot count keeps the block's warps (16 lanes: 16 warps, <= 907
# slots; 8 lanes: 9 warps, <= 807 slots)
SCHED_TUNE = {
    16: {"jrhs": ((6.0, 3.0, 588627), 550), "rhs": ((1.5, None, 405133), 550)},
    8: {"jrhs": ((2.0, 0.0, 509381), 400), "rhs": ((2.0, 1.0, 795782), 500)},
}
# shared memory of one block (227 KiB) and the warps per block the slot arrays
# allow, at most 16: at 16 lanes per cell (728 slots) 16 warps ran a 64^3 collapse
# in 32.5 s on GB300, 17 warps in 34.3 s and 19 warps (register-limited) in 33.3 s
SMEM_BLOCK = 232448
MAX_WARPS = 16
# lane widths whose slots are allocated bank by bank (allocate_banked)
BANKED = (16,)


def warps_per_block(G: int, nv: int) -> int:
    """Warps of the cooperative advance's block: as many as the cells' slot
    arrays fit in one block's shared memory (one block per SM), at most
    MAX_WARPS."""
    cells = (SMEM_BLOCK // 8) // nv
    return max(1, min(MAX_WARPS, cells // (32 // G)))


def generate(G: int, dag=None, limit="default", tune="default", banked="default"):
    """Programs jrhs and rhs for G lanes per cell: a dict with the encoded steps,
    the output operands, the slot count, the reserved constants and the warps
    per block.  ``banked``: allocate slots with ``allocate_banked`` within the
    slot count that keeps the block's warps (G = 16)."""
    dag = dag or ir_io.load()
    if limit == "default":
        limit = SCHED_LIMIT.get(G)
    if tune == "default":
        tune = SCHED_TUNE.get(G)
    built = {}
    pool = {0, 1, dbits(1.0), dbits(-1.0), dbits(-0.0)}
    funs = set()
    for kind in ("jrhs", "rhs"):
        P, out = build(dag, kind)
        lower(P)
        pool |= reserved_constants(P, out)
        funs |= device_constants(P, out)
        built[kind] = (P, out)
    # reserved slots: false/+0.0, true, 1, -1, -0 first, then the rest in order,
    # then the transcendentals of constants
    fixed = [0, 1, dbits(1.0), dbits(-1.0), dbits(-0.0)]
    rconst = fixed + sorted(pool - set(fixed))
    rfun = sorted(funs)
    res = {b: RES_BASE + i for i, b in enumerate(rconst)}
    res.update({f: RES_BASE + len(rconst) + j for j, f in enumerate(rfun)})
    first = RES_BASE + len(rconst) + len(rfun)
    if banked == "default":
        banked = G in BANKED
    # slot count (write sink included) that keeps the block's warps, one below the
    # block's whole shared memory
    cap = max(nv for nv in range(first, MAX_SLOTS) if warps_per_block(G, nv) == MAX_WARPS) - 1
    scheds = {}
    for kind, (P, out) in built.items():
        t, lim = (tune or {}).get(kind, (None, limit))
        scheds[kind] = schedule(P, out, G, jac=(kind == "jrhs"), limit=lim, first_scratch=first, tune=t,
                                banked=(res, cap) if banked else None)
    nv = max(sch.nv for sch, _ in scheds.values())
    if nv * 8 > 0xfff8:
        raise ValueError(f"{nv} slots do not fit the 16-bit byte offsets")
    progs = {}
    for kind, (P, out) in built.items():
        sch, _ = scheds[kind]
        st = stats(sch)
        sch.nv = nv  # one slot map (and one write sink, the last slot) for both programs
        words = encode(P, sch, res)

        def outop(r, negate=False):
            b, neg, ab = r
            if negate:
                neg = not neg
            op = P.nodes[b][0]
            v = res[P.nodes[b][1][0]] if op == "const" else res[P.nodes[b][1]] if op == "dconst" else sch.slot[b]
            return v | (OPF_NEG if neg else 0) | (OPF_ABS if ab else 0)

        progs[kind] = {"words": words, "rhs_out": [outop(r) for r in sch.outputs["rhs"]],
                       "nsteps": len(words) - PREFETCH_PAD, "stats": st}
        if "jac" in sch.outputs:  # E = -J, entry r * 15 + c
            progs[kind]["jac_out"] = [outop(r, negate=True) for r in sch.outputs["jac"]]
    return {"G": G, "nv": nv, "rconst": rconst, "rfun": rfun, "progs": progs, "warps": warps_per_block(G, nv)}


def shared_wavefronts(pr: dict) -> dict:
    """Shared-memory wavefronts of one encoded program's slot accesses, per half
    warp, by operand (X, Y, Z, D of the main word; A, B, C, D2 of the integer word),
    against one wavefront per access.  A 64-bit access of a half warp (one cell's
    G = 16 lanes) is conflict-free when its distinct slots lie in distinct bank
    pairs (slot mod 16: the cell's array base is uniform over the half warp);
    otherwise it takes as many wavefronts as the most-used bank pair holds distinct
    slots.  Accesses follow the interpreter: an FMA step loads X, Y, Z; exp, log
    and sqrt load Y, division X and Y; every non-idle step stores D; a step with
    integer nodes loads A, B, C and stores D2."""
    def wf(slots):
        by = collections.defaultdict(set)
        for s in slots:
            by[s % 16].add(s)
        return max(len(v) for v in by.values())

    def field(w, k):
        return ((w >> (16 * k)) & 0xffff) >> 3

    got, ideal = collections.Counter(), collections.Counter()
    for lanes in pr["words"][:pr["nsteps"]]:
        m0 = lanes[0][0]
        cls, flint = (m0 >> 48) & 7, (m0 >> 32) & FL_INT
        used = {C_FMA: "XYZD", C_DIV: "XYD"}.get(cls, "YD" if cls != C_NONE else "")
        acc = [(n, [field(m, "XYZD".index(n)) for m, _, _ in lanes]) for n in used]
        if flint:
            acc += [(n, [field(i, k) for _, i, _ in lanes]) for k, n in enumerate(("A", "B", "C", "D2"))]
        for n, slots in acc:
            got[n] += wf(slots)
            ideal[n] += 1
    return {"wavefronts": sum(got.values()), "ideal": sum(ideal.values()),
            "by_operand": {n: (got[n], ideal[n]) for n in sorted(got)}}


def stats(sch: Schedule) -> dict:
    cnt = collections.Counter(c for c, _, _ in sch.steps)
    cost = sum(STEP_COST.get(c, 0.0) for c, _, _ in sch.steps)
    return {"steps": len(sch.steps), "by_class": {str(k): v for k, v in sorted(cnt.items())},
            "fp64_slots": cost, "slots": sch.nv}


def emit_header(G: int, gen: dict, digest: str) -> str:
    lines = [
        "// Generated by warp_reactor_gb300/gen/coop.py from network.ir",
        f"// network.ir sha256 {digest}",
        f"// Vector programs of the network for {G} lanes per cell.",
        "#pragma once",
        "#include <stdint.h>",
        "",
        f"namespace wr {{ namespace coop{G} {{",
        f"constexpr int kG = {G};",
        f"constexpr int kNV = {gen['nv']};",
        f"constexpr int kNR = {len(gen['rconst'])};  // reserved constant slots from {RES_BASE}",
        f"constexpr int kNF = {len(gen['rfun'])};  // then the transcendentals of constants",
        f"constexpr int kWarps = {gen['warps']};  // warps per block: the slot arrays that fit in shared memory",
    ]
    for kind, pr in gen["progs"].items():
        st = pr["stats"]
        lines.append(f"constexpr int k{kind.upper()}Steps = {pr['nsteps']};  // {st['by_class']}, "
                     f"{st['fp64_slots']:.0f} FP64 issue slots, {st['steps']} steps before padding")
    lines.append("")
    lines.append("static __device__ const uint64_t kVConst[kNR] = {")
    cs = gen["rconst"]
    for i in range(0, len(cs), 4):
        lines.append("    " + ", ".join(f"0x{b:016x}ULL" for b in cs[i:i + 4]) + ",")
    lines.append("};")
    lines.append("// (class, argument bits): exp (2), log (3) or sqrt (4) of a constant")
    lines.append(f"static __device__ const ulonglong2 kVFun[{max(1, len(gen['rfun']))}] = {{")
    for c, b in gen["rfun"] or [(0, 0)]:
        lines.append(f"    {{{c}ULL, 0x{b:016x}ULL}},")
    lines.append("};")
    for kind, pr in gen["progs"].items():
        K = kind.upper()
        n = f"(k{K}Steps + {PREFETCH_PAD}) * kG"
        lines.append(f"static __device__ const ulonglong2 k{K}Prog[{n}] = {{")
        for lanes in pr["words"]:
            lines.append("    " + ", ".join(f"{{0x{m:x}ULL, 0x{i:x}ULL}}" for m, i, _ in lanes) + ",")
        lines.append("};")
        lines.append(f"static __device__ const uint64_t k{K}Lit[{n}] = {{")
        for lanes in pr["words"]:
            lines.append("    " + ", ".join(f"0x{l:x}ULL" for _, _, l in lanes) + ",")
        lines.append("};")
        lines.append(f"static __device__ const uint16_t k{K}Out[15] = {{" +
                     ", ".join(str(v) for v in pr["rhs_out"]) + "};")
        if "jac_out" in pr:
            lines.append(f"static __device__ const uint16_t k{K}Jac[225] = {{")
            jo = pr["jac_out"]
            for i in range(0, 225, 15):
                lines.append("    " + ", ".join(str(v) for v in jo[i:i + 15]) + ",")
            lines.append("};")
    lines.append(f"}} }}  // namespace wr::coop{G}")
    return "\n".join(lines) + "\n"


HERE = os.path.dirname(os.path.abspath(__file__))
GEN_DIR = os.path.join(os.path.dirname(HERE), "csrc", "generated")
LANES_PER_CELL = (8, 16, 32)


def emit_all(out_dir: str = GEN_DIR, ir_path: str = ir_io.DEFAULT_PATH) -> list:
    from .build_network import _write_if_changed
    dag = ir_io.load(ir_path)
    digest = ir_io.digest(ir_path)
    paths = []
    for G in LANES_PER_CELL:
        path = os.path.join(out_dir, f"coop_prog_g{G}.h")
        _write_if_changed(path, emit_header(G, generate(G, dag), digest))
        paths.append(path)
    return paths


if __name__ == "__main__":
    d = ir_io.load()
    for G in LANES_PER_CELL:
        g = generate(G, d)
        print(G, g["nv"], len(g["rconst"]), g["warps"], {k: v["stats"] for k, v in g["progs"].items()})
        if G == 16:
            print("  shared wavefronts per half warp:",
                  {k: {f: w[f] for f in ("wavefronts", "ideal")} for k, w in
                   ((k, shared_wavefronts(v)) for k, v in g["progs"].items())})
