"""The hard input sets that pin the oracle to the reference library on the
CPU, run through the GPU kernels against the same oracle on the same
inputs - so each GPU result equals the reference library's by the chain
GPU == oracle == reference:

* raw and boundary encodings (tests/test_oracle.py's _raw_and_boundary:
  uniform random words over the whole encoding space, then exponents moved
  next to the overflow and underflow thresholds) through the element
  kernels: FMA/ADD/SUB/MUL, division and square root, every attribute,
  every value and every element's flags;
* raw encodings and sums next to the overflow threshold
  (tests/test_reduce_oracle.py's _wide) through the reduction kernels,
  plain and segmented, every attribute;
* mutated programs (tests/test_seq_fuzz_differential.py's mutation: seeded
  bit flips in the opcode, register and rounding fields of arithmetic
  instructions) through the sequencer kernel, every output;
* mutated ODE segment programs (tests/test_bundles.py's mutation) through
  the trajectory kernel at 1, 8 and 32 threads a lane, states, kept states
  and flags segment by segment.
"""
import ctypes

import numpy as np
import pytest

import cftgb
import oracle_lib
import seq_util as su
from cftgb import workload as wl
from test_elem_gpu import device_run
from test_oracle import _raw_and_boundary
from test_reduce_gpu import _bind as _bind_reduce
from test_reduce_oracle import _wide

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_raw_and_boundary_encodings_through_element_kernels(gpu, oracle, fmt):
    n = 12000
    a, b, c = _raw_and_boundary(fmt, n, 131 + fmt)
    for kind, op in ((0, 0), (0, 1), (0, 2), (0, 3), (1, 0), (2, 0)):
        for rnd in range(5):
            d, lf, acc = device_run(gpu, kind, fmt, op, rnd, a, b, c)
            rd, rlf, racc = oracle.run(kind, fmt, op, rnd, a, b, c)
            vbad = np.nonzero((d != rd).any(1))[0]
            fbad = np.nonzero(lf != rlf)[0]
            assert vbad.size == 0 and fbad.size == 0, (kind, op, rnd, vbad[:4], fbad[:4])
            assert acc & 0x1F == racc, (kind, op, rnd)


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_wide_encodings_and_near_overflow_sums_through_reductions(gpu, oracle, fmt):
    L = cftgb.lib()
    _bind_reduce(L, oracle)
    W = wl.words(fmt)
    for op in (24, 25, 28, 29, 31):
        for n in (2, 7, 64, 513, 9000, 70000):
            a, b = _wide(fmt, n, 5000 * fmt + n)
            for rnd in range(5):
                d, fl = np.zeros(W, np.uint32), ctypes.c_uint32()
                assert L.cft_reduce(gpu, op, fmt, rnd, a.ctypes.data,
                                    b.ctypes.data if op == 25 else None, d.ctypes.data, n,
                                    ctypes.byref(fl), None) == 0
                rd, rfl = np.zeros(W, np.uint32), ctypes.c_uint32()
                assert oracle.L.sfp_reduce(fmt, op, rnd, a.ctypes.data, b.ctypes.data,
                                           rd.ctypes.data, n, ctypes.byref(rfl)) == 0
                assert np.array_equal(d, rd) and fl.value == rfl.value, (op, n, rnd)
            # every value next to the overflow threshold
            t = n - n // 2
            a2, b2 = a[n // 2:].copy(), b[n // 2:].copy()
            d, fl = np.zeros(W, np.uint32), ctypes.c_uint32()
            assert L.cft_reduce(gpu, op, fmt, 0, a2.ctypes.data,
                                b2.ctypes.data if op == 25 else None, d.ctypes.data, t,
                                ctypes.byref(fl), None) == 0
            rd, rfl = np.zeros(W, np.uint32), ctypes.c_uint32()
            assert oracle.L.sfp_reduce(fmt, op, 0, a2.ctypes.data, b2.ctypes.data, rd.ctypes.data,
                                       t, ctypes.byref(rfl)) == 0
            assert np.array_equal(d, rd) and fl.value == rfl.value, (op, t, "near max")
        # segmented, over wide encodings
        for seg in (1, 3, 32, 96, 1024):
            m = 4096 // seg
            n = m * seg                       # whole segments
            a, b = _wide(fmt, n, 777 + fmt + seg)
            d, fl = np.zeros((m, W), np.uint32), ctypes.c_uint32()
            assert L.cft_reduce_seg(gpu, op, fmt, 3, a.ctypes.data,
                                    b.ctypes.data if op == 25 else None, d.ctypes.data, n, seg,
                                    ctypes.byref(fl), None) == 0
            rd, rfl = np.zeros((m, W), np.uint32), ctypes.c_uint32()
            assert oracle.L.sfp_reduce_seg(fmt, op, 3, a.ctypes.data, b.ctypes.data,
                                           rd.ctypes.data, n, seg, ctypes.byref(rfl)) == 0
            assert np.array_equal(d, rd) and fl.value == rfl.value, (op, seg)


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


def _mutate(img, sites, rng):
    img = img.copy()
    for _ in range(int(rng.integers(1, 4))):
        off = sites[int(rng.integers(0, len(sites)))]
        bit = int(rng.choice([*range(0, 24), 24, 25, 26]))   # op, rd/ra/rb/rc, rnd
        img[off + bit // 8] ^= np.uint8(1 << (bit % 8))
    return img


def test_mutated_programs_through_the_sequencer_kernel(gpu, oracle):
    rng = np.random.default_rng(99)
    ran, bad = 0, []
    for path in su.cases():
        case = su.load(path)
        sites = _arith_sites(case["image"])
        if not sites:
            continue
        for _ in range(12):
            m = dict(case)
            m["image"] = _mutate(case["image"], sites, rng)
            got = su.run_gpu(gpu, m)
            want = su.run_oracle(oracle, m)
            if isinstance(got, int):          # the loader refused it (as the reference's does)
                continue
            assert want is not None, path.stem
            diff = [k for k in ("deposits", "counts", "lane_flags", "scratch_out")
                    if not np.array_equal(np.asarray(got[k]).reshape(np.shape(want[k])), want[k])]
            diff += [k for k in ("flags", "status") if int(got[k]) != int(want[k])]
            if diff:
                bad.append((path.stem, diff))
            ran += 1
    assert not bad, bad[:5]
    assert ran > 150, ran


@pytest.mark.parametrize("G", ["1", "8", "32", "8c", "32c"])
@pytest.mark.parametrize("key,fmt,slots,base", [("l63", 3, 3, 1.0), ("hh", 3, 4, None),
                                                ("l96", 2, 40, 8.0)], ids=["l63", "hh", "l96"])
def test_mutated_ode_programs_through_the_trajectory_kernel(gpu, oracle, monkeypatch, G, key, fmt,
                                                            slots, base):
    import bench_suites as suites
    from test_traj_gpu import _traj
    monkeypatch.setenv("CFTG_LANE_THREADS", G.rstrip("c"))
    monkeypatch.setenv("CFTG_LANE_COOP", "1" if G.endswith("c") else "0")
    z = np.load(su.GOLD / "odes.npz")
    img0, bank = z[key + "_image"].copy(), z[key + "_bank"].copy()
    W = wl.words(fmt)
    lanes = 9
    if base is None:
        init = suites.hh_init(lanes, 9)
    else:
        init, _ = suites.ode_lanes(key, fmt, lanes, slots, base, (100, 100), 100, 3)
    sites = _arith_sites(img0)
    rng = np.random.default_rng(70 + fmt)
    L = cftgb.lib()
    compared = 0
    for _ in range(8 if key != "l96" else 3):
        img = _mutate(img0, sites, rng)
        prog = ctypes.c_void_p()
        if L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)) != 0:
            continue
        L.cft_program_free(prog)
        segs = [1 + (i % 3) for i in range(lanes)]
        final, snaps, lf, fl, st = _traj(gpu, img, bank, init.copy(), segs, 1, 3)
        snaps = snaps.reshape(lanes, 3, slots, W)
        acc = 0
        for i in range(lanes):
            s = init[i * slots:(i + 1) * slots].copy()
            for k in range(segs[i]):
                out = np.zeros_like(s)
                A = oracle_lib.SeqArgs()
                a = np.zeros((1, W), np.uint32)
                A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
                A.scratch_in, A.scratch_out, A.depth = s.ctypes.data, out.ctypes.data, 256
                assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
                acc |= A.flags_out
                s = out
                assert np.array_equal(snaps[i, k], s), (key, G, i, k)
            assert np.array_equal(final[i * slots:(i + 1) * slots], s), (key, G, i)
        assert fl == acc, (key, G)
        compared += 1
    assert compared >= 2, compared
