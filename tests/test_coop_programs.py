"""The cooperative advance's generated vector programs, checked on the CPU.

``gen/coop.py`` turns the network DAG (with the burn_state_from_y prologue) into
steps of G lanes.  This test executes those steps exactly as the device does --
every lane gathers its operands (slots of the cell's own array, the lane's literal
XOR-ed into the second operand), then every lane stores its result, one step at a
time -- with the oracle's own exp/log, then gathers E = -J into the matrix slots
from the Jacobian output table, and requires the Jacobian and the RHS to equal the
oracle's jacobian(y) / rhs(y) bit for bit.  It also checks the schedule's hazards
(no lane reads a slot that another lane writes in the same step), that no step
writes a reserved constant, and the slot map: the RHS-only program leaves the
matrix slots (the LU factors) alone, and the Jacobian program's kept values lie
above them, so the gather reads no slot it writes.
"""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

from warp_reactor_gb300.gen import coop, ir_io

C_NONE, C_FMA, C_EXP, C_LOG, C_SQRT, C_DIV = range(6)
I_SEL, I_LE, I_LT, I_SGN = range(4)
SIGN = 1 << 63
ABS = SIGN - 1


def d(u):
    return struct.unpack("<d", struct.pack("<Q", u))[0]


def u(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def fetch(V, op):
    """An output operand: slot | negate | absolute value."""
    v = V[op & 0xfff]
    if op & coop.OPF_ABS:
        v &= ABS
    if op & coop.OPF_NEG:
        v ^= SIGN
    return v


def fma(a, b, c):
    """fma(a, b, c) with one rounding.  The generated forms have an exact product
    (a factor +-1) or an addend -0; other operands are rounded exactly through
    fractions (finite values only)."""
    if u(c) == u(-0.0):
        return a * b
    if b == 1.0:
        return a + c
    if b == -1.0:
        return c - a
    if a == 1.0:
        return b + c
    assert all(math.isfinite(v) for v in (a, b, c))
    r = Fraction(a) * Fraction(b) + Fraction(c)
    return float(r) if r != 0 else (a * b + c)


def mods(v, fl):
    if fl & coop.FL_ABS:
        v &= ABS
    if fl & coop.FL_NEG:
        v ^= SIGN
    return v


def ble(a, b):
    fa, fb = d(a), d(b)
    return int(fa <= fb)


def run(words, V, nres, oracle, written=None):
    sink = len(V) - 1
    reserved = set(range(coop.RES_BASE, coop.RES_BASE + nres))  # constants and transcendentals of constants
    for lanes in words:
        reads, writes, results = set(), set(), []
        for mw, iw, lit in lanes:
            f = [(mw >> (16 * k)) & 0xffff for k in range(4)]
            cls = f[3] & 7
            zfl = f[2] & 7
            if cls != C_NONE:
                xa, ya = f[0] >> 3, f[1] >> 3
                if cls == C_FMA:
                    assert f[0] & 7 == 0 and f[1] & 7 == 0, "flags on an FMA operand"
                    za = f[2] >> 3
                    reads.update((xa, ya, za))
                    r = fma(d(V[xa]), d(V[ya] ^ lit), d(V[za]))
                else:
                    reads.add(ya)
                    y = mods(V[ya] ^ lit, f[1])
                    if cls == C_DIV:
                        reads.add(xa)
                        x = mods(V[xa], f[0])
                        num, den = (d(y), d(x)) if f[1] & coop.FL_SWAP else (d(x), d(y))
                        if den != 0:
                            r = num / den
                        else:
                            r = (math.copysign(math.inf, num) * math.copysign(1, den) if num != 0 and num == num
                                 else float("nan"))
                    elif cls == C_EXP:
                        r = oracle.exp(d(y))
                    elif cls == C_LOG:
                        r = oracle.log(d(y))
                    else:
                        r = math.sqrt(d(y)) if d(y) >= 0 else float("nan")
                results.append((f[3] >> 3, u(r)))
            if zfl & coop.FL_INT:
                g = [(iw >> (16 * k)) & 0xffff for k in range(4)]
                A, B, C = (V[g[k] >> 3] for k in range(3))
                reads.update(g[k] >> 3 for k in range(3))
                iop = g[3] & 3
                r = B if A != 0 else C
                if zfl & coop.FL_SPECIAL:
                    if iop == I_LE:
                        r = ble(A, B)
                    elif iop == I_LT:
                        r = int(d(A) < d(B))
                    elif iop == I_SGN:
                        r = (A & ABS) if g[3] & coop.FL_SABS else (A ^ SIGN)
                else:
                    assert iop == I_SEL, "comparison or sign op in a step not flagged for them"
                results.append((g[3] >> 3, r))
        for dst, r in results:
            assert dst == sink or dst not in reads, f"slot {dst} written and read in one step"
            assert dst == sink or dst not in writes, f"slot {dst} written twice in one step"
            assert dst not in reserved, f"reserved slot {dst} written"
            writes.add(dst)
            if written is not None and dst != sink:
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
    ys = states(6, 11 + G)
    # plus the reference's initial cell (the first burn's y)
    c0 = oracle_port.make_collapse_state()
    ys = np.vstack([ys, np.concatenate([c0["xn"], [c0["e"]]])])
    nres = len(gen["rconst"])
    for y in ys:
        J_o = oracle_port.jac(y)
        f_o = oracle_port.rhs(y)
        for kind in ("jrhs", "rhs"):
            pr = gen["progs"][kind]
            V = [0x7ff4000000000000] * gen["nv"]  # signalling-NaN garbage: every read slot must be written
            for i, b in enumerate(gen["rconst"]):
                V[coop.RES_BASE + i] = b
            fn = {C_EXP: oracle_port.exp, C_LOG: oracle_port.log, C_SQRT: math.sqrt}
            for j, (cls, b) in enumerate(gen["rfun"]):  # the kernel's per-launch evaluation
                V[coop.RES_BASE + nres + j] = u(fn[cls](d(b)))
            for k in range(15):
                V[coop.Y_BASE + k] = u(y[k])
            written = set()
            run(pr["words"], V, nres + len(gen["rfun"]), oracle_port, written)
            f = np.array([d(fetch(V, o)) for o in pr["rhs_out"]])
            assert same(f, f_o), (G, kind)
            assert all((o & 0xfff) >= coop.E_SLOTS for o in pr["rhs_out"])
            if kind == "jrhs":
                jac = pr["jac_out"]
                assert len(jac) == 225
                assert all((o & 0xfff) >= coop.E_SLOTS for o in jac)
                for i in range(225):  # the kernel's gather: E = -J
                    V[i] = fetch(V, jac[i])
                J = -np.array([d(V[i]) for i in range(225)]).reshape(15, 15)
                assert same(J, J_o), G
            else:
                assert not any(w < coop.E_SLOTS for w in written), "RHS program writes a matrix slot"


@pytest.mark.parametrize("G", [8, 16, 32])
def test_program_shape(programs, G):
    """Byte offsets fit the 16-bit fields and a block's shared memory holds the
    cells' slot arrays; every step names one class and one pair of step flags for
    all lanes; steps come in groups of four, followed by idle prefetch padding."""
    gen = programs[G]
    assert gen["nv"] * 8 <= 0xfff8
    assert gen["warps"] * (32 // G) * gen["nv"] * 8 <= coop.SMEM_BLOCK
    for pr in gen["progs"].values():
        words = pr["words"]
        assert pr["nsteps"] % coop.STEP_ALIGN == 0
        assert len(words) == pr["nsteps"] + coop.PREFETCH_PAD
        assert all(w == (0, 0, 0) for lanes in words[pr["nsteps"]:] for w in lanes)
        for lanes in words:
            assert len({(mw >> 48) & 7 for mw, _, _ in lanes}) == 1
            assert len({(mw >> 32) & 7 for mw, _, _ in lanes}) == 1


def test_banked_slot_map(programs):
    """At 16 lanes per cell the slots are allocated bank by bank: within the slot
    count that keeps 16 warps per block, the interpreter's shared accesses take at
    most 20 % more wavefronts than one per access (the linear scan took 95 % more),
    and every step's stores go to distinct bank pairs but for a few."""
    gen = programs[16]
    assert gen["nv"] <= 907 and gen["warps"] == coop.MAX_WARPS
    for pr in gen["progs"].values():
        w = coop.shared_wavefronts(pr)
        assert w["wavefronts"] <= 1.2 * w["ideal"], w
        stores, ideal = w["by_operand"]["D"]
        assert stores <= 1.25 * ideal, w
