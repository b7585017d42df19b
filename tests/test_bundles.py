"""The bundle schedule (G threads a lane, cftg_program_schedule) replayed on
the host: each bundle's operations read their operands, then all write,
with the oracle's arithmetic (sfp_compute). The state and flags after a run
must equal the oracle's own sequencer (sfp_seq_run) on the same lanes, for
every G - a check of the scheduler's dependence rules with no GPU."""
import ctypes

import numpy as np
import pytest

import cftgb
import oracle_lib
import seq_util as su
import bench_suites as suites
from cftgb import workload as wl

NOP = (1 << 64) - 1


def schedule(img, G):
    L = cftgb.lib()
    vp = ctypes.c_void_p
    L.cftg_program_schedule.argtypes = [vp, ctypes.c_size_t, ctypes.c_uint32, vp, vp, vp, vp,
                                        ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    nb = ctypes.c_size_t()
    st = L.cftg_program_schedule(img.ctypes.data, img.size, G, None, None, None, None, 0,
                                 ctypes.byref(nb))
    if st:
        return None
    n = nb.value
    ops = np.zeros(n * G, np.uint64)
    ctl = np.zeros(n, np.uint32)
    arg = np.zeros(n, np.uint32)
    match = np.zeros(n, np.int32)
    assert L.cftg_program_schedule(img.ctypes.data, img.size, G, ops.ctypes.data, ctl.ctypes.data,
                                   arg.ctypes.data, match.ctypes.data, n, ctypes.byref(nb)) == 0
    return ops.reshape(n, G), ctl, arg, match


def replay(oracle, sched, fmt, bank, block, reach, W):
    """One run of one lane through the schedule; returns (scratch, flags).
    Locations: registers 0..31, scratch slots 32.., renamed values after."""
    ops, ctl, arg, match = sched
    loc = np.zeros((4096, W), np.uint32)
    loc[32:32 + len(block)] = block
    kons = bank.view(np.uint32).reshape(-1, W) if bank is not None and bank.size else None
    flags = 0
    b, stack = 0, []
    out = np.zeros(W, np.uint32)
    fl = ctypes.c_uint32()
    while b < len(ctl):
        if ctl[b] == 0:
            writes = []
            for u in ops[b]:
                u = int(u)
                if u == NOP:
                    continue
                dest, ia, ib, ic = (u >> 16) & 0xFFF, (u >> 28) & 0xFFF, (u >> 40) & 0xFFF, (u >> 52) & 0xFFF
                if (u >> 14) & 1:                     # MOVE
                    writes.append((dest, loc[ia].copy()))
                    continue
                vals = [np.ascontiguousarray(kons[i] if (u >> (11 + k)) & 1 else loc[i])
                        for k, i in enumerate((ia, ib, ic))]
                if (u >> 15) & 1:                     # a NEG folded into operand c
                    vals[2] = vals[2].copy()
                    vals[2][W - 1] ^= np.uint32(0x80000000)
                assert oracle.L.sfp_compute(fmt, u & 0xFF, (u >> 8) & 7, vals[0].ctypes.data,
                                            vals[1].ctypes.data, vals[2].ctypes.data,
                                            out.ctypes.data, ctypes.byref(fl)) == 0
                flags |= fl.value
                writes.append((dest, out.copy()))
            for where, v in writes:
                loc[where] = v
            b += 1
        elif ctl[b] == 1:
            if arg[b] == 0:
                b = int(match[b]) + 1
            else:
                stack.append([b + 1, int(arg[b])])
                b += 1
        elif ctl[b] == 2:
            stack[-1][1] -= 1
            if stack[-1][1] > 0:
                b = stack[-1][0]
            else:
                stack.pop()
                b += 1
        else:
            break
    return loc[32:32 + reach], flags


ODES = [("l63", 3, 3, 1.0), ("l96", 2, 40, 8.0), ("hh", 3, 4, None)]


@pytest.mark.parametrize("key,fmt,slots,base", ODES, ids=[o[0] for o in ODES])
@pytest.mark.parametrize("G", [1, 2, 4, 8, 32])
def test_schedule_replay_equals_sequencer(oracle, key, fmt, slots, base, G):
    oracle.L.sfp_compute.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4 + [
        ctypes.POINTER(ctypes.c_uint32)]
    z = np.load(su.GOLD / "odes.npz")
    img, bank = z[key + "_image"].copy(), z[key + "_bank"].copy()
    sched = schedule(img, G)
    assert sched is not None
    ops = sched[0]
    assert (ops != np.uint64(NOP)).sum(axis=1).max() <= G
    W = wl.words(fmt)
    if base is None:
        init = suites.hh_init(1, 9)
    else:
        init, _ = suites.ode_lanes(key, fmt, 1, slots, base, (100, 100), 100, 3)
    got, gflags = replay(oracle, sched, fmt, bank, init, 256, W)
    out = np.zeros_like(init)
    A = oracle_lib.SeqArgs()
    a = np.zeros((1, W), np.uint32)
    A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
    A.scratch_in, A.scratch_out, A.depth = init.ctypes.data, out.ctypes.data, 256
    assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
    assert np.array_equal(got[:slots], out), f"{key} G={G}"
    assert gflags == A.flags_out


def test_schedule_parallelism():
    """The schedule actually finds parallel work: Lorenz-96 (40 independent
    components) fills wide bundles; and a program outside the scheduled set
    (one that deposits) is refused."""
    z = np.load(su.GOLD / "odes.npz")
    img = z["l96_image"].copy()
    n1 = len(schedule(img, 1)[1])
    n32 = len(schedule(img, 32)[1])
    assert n32 * 8 < n1, (n1, n32)
    dep = next(p for p in su.cases() if su.header(su.load(p)["image"])["maxdep"] > 0)
    assert schedule(su.load(dep)["image"].copy(), 4) is None


def _arith_sites(img):
    hd = su.header(img)
    esz = (4, 8, 16, 32)[hd["prec"]]
    base = 32 + (0 if hd["flags"] & 1 else hd["n_consts"] * esz)
    out = []
    for i in range(hd["n_insns"]):
        w = int.from_bytes(bytes(img[base + 8 * i:base + 8 * i + 8]), "little")
        if not (w >> 27) & 0x1F:              # no constant flags, kx or ctrl
            out.append(base + 8 * i)
    return out


@pytest.mark.parametrize("key,fmt,slots,base,count", [
    ("l63", 3, 3, 1.0, 24), ("hh", 3, 4, None, 24), ("l96", 2, 40, 8.0, 6)],
    ids=["l63", "hh", "l96"])
def test_schedule_replay_on_mutated_programs(oracle, key, fmt, slots, base, count):
    """Seeded bit flips in the opcode, register and rounding fields of the
    ODE programs' arithmetic instructions give dependence patterns the
    shipped programs do not have (reads before writes, overwritten operands,
    reused registers); for every mutant the sequencer accepts and the
    scheduler takes, the replay at G = 1, 4 and 32 equals the sequencer."""
    oracle.L.sfp_compute.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4 + [
        ctypes.POINTER(ctypes.c_uint32)]
    z = np.load(su.GOLD / "odes.npz")
    img0, bank = z[key + "_image"].copy(), z[key + "_bank"].copy()
    W = wl.words(fmt)
    if base is None:
        init = suites.hh_init(1, 9)
    else:
        init, _ = suites.ode_lanes(key, fmt, 1, slots, base, (100, 100), 100, 3)
    sites = _arith_sites(img0)
    rng = np.random.default_rng(7 + fmt)
    compared = 0
    for _ in range(count):
        img = img0.copy()
        for _ in range(int(rng.integers(1, 4))):
            off = sites[int(rng.integers(0, len(sites)))]
            bit = int(rng.choice([*range(0, 24), 24, 25, 26]))
            img[off + bit // 8] ^= np.uint8(1 << (bit % 8))
        out = np.zeros_like(init)
        A = oracle_lib.SeqArgs()
        a = np.zeros((1, W), np.uint32)
        A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
        A.scratch_in, A.scratch_out, A.depth = init.ctypes.data, out.ctypes.data, 256
        if oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) != 0:
            continue
        for G in (1, 4, 32):
            sched = schedule(img, G)
            if sched is None:
                break
            got, gflags = replay(oracle, sched, fmt, bank, init, 256, W)
            assert np.array_equal(got[:slots], out), (key, G)
            assert gflags == A.flags_out, (key, G)
            compared += 1
    assert compared >= count, (key, compared)


# A stretch that stresses the schedule's two rewrites (a NEG folded into the
# operand c that reads it; a stretch-end MOVE folded into its value's
# producer): a NEG whose operand register is overwritten before the
# operation that reads the NEG; NEGs read as operands a and b (not folded)
# and as c; a NEG result that is also the stretch's final value of its
# register; a register read (its value from before the stretch) after the
# producer of its final value in program order; a value stored to two
# slots; a slot loaded after a store to another slot.
HAZARDS = """
.format   fp64
.deposits 0
.scratch  in 3
.scratch  out 3
ldl  r1, 0
ldl  r2, 1
ldl  r6, 2
repeat 5
  neg  r3, r1
  add  r1, r1, r2
  fma  r4, r2, r2, r3
  neg  r5, r4
  mul  r7, r5, r3
  fma  r8, r7, r1, r5
  neg  r9, r8
  fma  r2, r9, r6, r9
  sub  r6, r6, r2
  fma  r10, r6, r2, r6
  neg  r6, r10
  stl  r8, 2
  stl  r8, 0
  ldl  r11, 1
  fma  r1, r11, r3, r1
endrep
stl  r1, 0
stl  r2, 1
halt
"""


@pytest.mark.parametrize("G", [1, 2, 4, 8, 32])
def test_schedule_rewrites_keep_the_sequencer_s_values(oracle, G):
    from cftgb import asm
    oracle.L.sfp_compute.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4 + [
        ctypes.POINTER(ctypes.c_uint32)]
    img = np.frombuffer(asm.assemble(HAZARDS, "hazards.cfta"), np.uint8).copy()
    sched = schedule(img, G)
    assert sched is not None
    W = 2
    rng = np.random.default_rng(G)
    for trial in range(4):
        vals = rng.uniform(-2.0, 2.0, size=3)
        init = np.array([wl.from_int(wl.encode_double(1, float(v)), W) for v in vals], np.uint32)
        got, gflags = replay(oracle, sched, 1, None, init, 256, W)
        out = np.zeros_like(init)
        A = oracle_lib.SeqArgs()
        a = np.zeros((1, W), np.uint32)
        A.a, A.n = a.ctypes.data, 1
        A.scratch_in, A.scratch_out, A.depth = init.ctypes.data, out.ctypes.data, 256
        assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
        assert np.array_equal(got[:3], out), (G, trial)
        assert gflags == A.flags_out


def test_schedule_rewrites_fold_the_ode_negations():
    """Lorenz-63's step: the NEGs leave the chains that read them and the
    stretch's end MOVEs are gone, so at 8 threads a lane a step is at most
    18 bundles (25 without the rewrites); no micro-operation keeps a NEG of
    a value only a folded read used."""
    z = np.load(su.GOLD / "odes.npz")
    ops, ctl, _, _ = schedule(z["l63_image"].copy(), 8)
    assert len(ctl) <= 18, len(ctl)
    words = [int(u) for u in ops.reshape(-1) if int(u) != NOP]
    assert any((u >> 15) & 1 for u in words)
