"""The cooperative advance's generated vector programs, checked on the CPU.

``gen/coop.py`` turns the network DAG (with the burn_state_from_y prologue) into
steps of G lanes.  This test executes those steps exactly as the device does --
every lane gathers its operands, then every lane stores its result, one step at a
time -- with the oracle's own exp/log, then gathers E = -J into the matrix slots
from the Jacobian output table, and requires the Jacobian and the RHS to equal the
oracle's jacobian(y) / rhs(y) bit for bit.  It also checks the schedule's hazards
(no lane reads a slot that another lane writes in the same step) and the slot
map: the RHS-only program leaves the matrix slots (the LU factors) alone, and the
Jacobian program's kept values lie above them, so the gather reads no slot it
writes.
"""
import math
import struct

import numpy as np
import pytest

from warp_reactor_gb300.gen import coop, ir_io

C_NONE, C_FMA, C_EXP, C_LOG, C_SQRT, C_DIV = range(6)
I_SEL, I_LE, I_LT = range(3)
SIGN = 1 << 63
ABS = SIGN - 1


def d(u):
    return struct.unpack("<d", struct.pack("<Q", u))[0]


def u(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def fetch(V, C, op):
    v = C[op & 0xfff] if op & 0x1000 else V[op & 0xfff]
    if op & 0x4000:
        v &= ABS
    if op & 0x2000:
        v ^= SIGN
    return v


def fma_special(a, b, c, one, mzero):
    """fma(a, b, c) for the operand forms the generator emits: a*b with c = -0,
    a + c with b = 1 (a single rounding either way, so plain Python floats)."""
    if u(c) == mzero:
        return a * b
    assert u(b) == one
    return a + c


def run(words, V, C, oracle, one, mzero, written=None):
    for lanes in words:
        reads, writes, results = set(), set(), []
        for mw, iw in lanes:
            cls = (mw >> 60) & 7
            if cls != C_NONE:
                ops = [(mw >> (16 * k)) & 0xffff for k in range(3)]
                reads.update(o & 0xfff for o in ops if not o & 0x1000)
                a, b, c = (d(fetch(V, C, o)) for o in ops)
                if cls == C_FMA:
                    r = fma_special(a, b, c, one, mzero)
                elif cls == C_EXP:
                    r = oracle.exp(a)
                elif cls == C_LOG:
                    r = oracle.log(a)
                elif cls == C_SQRT:
                    r = math.sqrt(a) if a >= 0 else float("nan")
                else:
                    r = a / b if b != 0 else (math.copysign(math.inf, a) * math.copysign(1, b) if a != 0 and a == a
                                              else float("nan"))
                results.append(((mw >> 48) & 0xfff, u(r)))
            if mw >> 63:
                iop = iw >> 60
                ops = [(iw >> (16 * k)) & 0xffff for k in range(3)]
                reads.update(o & 0xfff for o in ops if not o & 0x1000)
                A, B, Cc = (fetch(V, C, o) for o in ops)
                fa, fb = d(A), d(B)
                r = {I_LE: int(fa <= fb), I_LT: int(fa < fb), I_SEL: B if A else Cc}[iop]
                results.append(((iw >> 48) & 0xfff, r))
        sink = len(V) - 1
        for dst, r in results:
            assert dst == sink or dst not in reads, f"slot {dst} written and read in one step"
            assert dst == sink or dst not in writes, f"slot {dst} written twice in one step"
            writes.add(dst)
            if written is not None and dst != len(V) - 1:
                written.add(dst)
            V[dst] = r


def same(a, b):
    """Bit-identical, except that a NaN matches any NaN (x86 and the GPU write
    different default-NaN patterns; integration states never reach NaN)."""
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return bool(((a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))).all())


def states(n, seed):
    rng = np.random.default_rng(seed)
    X = 10.0 ** rng.uniform(-30, 2, size=(n, 14))
    e = 10.0 ** rng.uniform(9, 12, size=(n, 1))
    return np.hstack([X, e])


@pytest.fixture(scope="module")
def programs():
    dag = ir_io.load()
    return {G: coop.generate(G, dag) for G in (8, 16, 32)}


@pytest.mark.parametrize("G", [8, 16, 32])
def test_programs_equal_oracle(programs, oracle_port, G):
    gen = programs[G]
    C = list(gen["consts"])
    one, mzero = u(1.0), u(-0.0)
    ys = states(6, 11 + G)
    # plus the reference's initial cell (the first burn's y)
    c0 = oracle_port.make_collapse_state()
    ys = np.vstack([ys, np.concatenate([c0["xn"], [c0["e"]]])])
    for y in ys:
        J_o = oracle_port.jac(y)
        f_o = oracle_port.rhs(y)
        for kind in ("jrhs", "rhs"):
            pr = gen["progs"][kind]
            V = [0] * gen["nv"]
            for k in range(15):
                V[coop.Y_BASE + k] = u(y[k])
            written = set()
            run(pr["words"], V, C, oracle_port, one, mzero, written)
            f = np.array([d(fetch(V, C, o)) for o in pr["rhs_out"]])
            assert same(f, f_o), (G, kind)
            assert all(o & 0x1000 or (o & 0xfff) >= coop.E_SLOTS for o in pr["rhs_out"])
            if kind == "jrhs":
                jac = pr["jac_out"]
                assert len(jac) == 225
                assert all(o & 0x1000 or (o & 0xfff) >= coop.E_SLOTS for o in jac)
                for i in range(225):  # the kernel's gather: E = -J
                    V[i] = fetch(V, C, jac[i])
                J = -np.array([d(V[i]) for i in range(225)]).reshape(15, 15)
                assert same(J, J_o), G
            else:
                assert not any(w < coop.E_SLOTS for w in written), "RHS program writes a matrix slot"


@pytest.mark.parametrize("G", [8, 16, 32])
def test_program_shape(programs, G):
    """Slots fit the 12-bit field and a block's shared memory; every step's
    main word names one class for all lanes."""
    gen = programs[G]
    assert gen["nv"] <= 4096 and len(gen["consts"]) <= 4096
    ncpad = (len(gen["consts"]) + 1) & ~1
    assert (ncpad + gen["warps"] * (32 // G) * gen["nv"]) * 8 <= coop.SMEM_BLOCK
    for pr in gen["progs"].values():
        for lanes in pr["words"]:
            assert len({(mw >> 60) for mw, _ in lanes}) == 1
