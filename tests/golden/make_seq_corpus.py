"""Generate tests/golden/seq_corpus/<fmt>.npz: the first corpus of the
reference's sequencer differential (host/tests/seq_check.py, its main
loop's first two arms: random valid programs from the golden model's
generator `seq.random_program`, alternately with the extended opcode pool -
IMUL and kx-indexed constants over a deep bank - and corrupted 30 % of the
time by seq_check's own `corrupt`), with the golden model's results
(`seq.run`) or its refusal. Run where the reference tree is present:

    python tests/golden/make_seq_corpus.py [REFERENCE_TREE]   # or CFT_REFERENCE

The draw follows seq_check's main loop for a trial (the same calls, the
same seed per format: 17 ^ (width * 7919)), so the programs are the ones
seq_check compares; the expected values are the golden model's, as
seq_check's are. Each format's file holds, per trial: the image, whether
the model refuses it, and for the others the lane count n, the a/b/c
streams, the deposits, the per-lane deposit counts, the flags and the
status word. Variable-length fields are concatenated with offset arrays.
"""
import random
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = ROOT / "tests" / "golden" / "seq_corpus"
TRIALS = 240


def words(v, W):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(W)]


def main(ref):
    ref = Path(ref)
    sys.path.insert(0, str(ref / "python"))
    sys.path.insert(0, str(ref / "host" / "tests"))
    import seq_check as sc
    OUT.mkdir(parents=True, exist_ok=True)
    for name in ("fp32", "fp64", "fp128", "fp256"):
        fmt = sc.FORMATS[name]
        W = fmt.width // 32
        rng = random.Random(17 ^ (fmt.width * 7919))
        images, refused, ns, streams, deps, dep_off, counts, flags, status = \
            [], [], [], [], [], [0], [], [], []
        for trial in range(TRIALS):
            ext = (trial % 2) == 1
            insns, consts = sc.seq.random_program(fmt, rng, extended=ext)
            maxdep = rng.choice([0, 1, 2, 4])
            if rng.random() < 0.3:
                insns, _ = sc.corrupt(insns, rng)
            try:
                prog = sc.mprog(fmt, insns, consts, maxdep)
            except sc.seq.ProgramError:
                # serialised without the constructor that refused it, as
                # seq_check does
                bogus = sc.seq.Program.__new__(sc.seq.Program)
                bogus.fmt, bogus.insns = fmt, insns
                bogus.consts, bogus.max_deposits = consts, maxdep
                bogus.flags = 0
                bogus.n_scratch_in = bogus.n_scratch_out = 0
                bogus._n_consts = len(consts)
                images.append(np.frombuffer(bogus.to_bytes(), np.uint8))
                refused.append(1)
                ns.append(0)
                dep_off.append(dep_off[-1])
                flags.append(0)
                status.append(0)
                continue
            n = rng.choice([1, 2, 63, 64, 65, 100, 129])
            a = sc.seq.random_inputs(fmt, rng, n)
            b = sc.seq.random_inputs(fmt, rng, n)
            c = sc.seq.random_inputs(fmt, rng, n)
            want = sc.mrun(prog, a, b, c)
            images.append(np.frombuffer(prog.to_bytes(), np.uint8))
            refused.append(0)
            ns.append(n)
            for s in (a, b, c):
                streams.extend(words(v, W) for v in s)
            deps.extend(words(v, W) for v in want.deposits)
            dep_off.append(len(deps))
            counts.extend(want.counts)
            flags.append(want.flags)
            status.append(want.status)
        img_off = np.cumsum([0] + [len(x) for x in images])
        np.savez_compressed(
            OUT / f"{name}.npz",
            images=np.concatenate(images), img_off=img_off.astype(np.int64),
            refused=np.array(refused, np.uint8), n=np.array(ns, np.int64),
            streams=np.array(streams, np.uint32).reshape(-1, W),
            deposits=np.array(deps, np.uint32).reshape(-1, W),
            dep_off=np.array(dep_off, np.int64), counts=np.array(counts, np.uint32),
            flags=np.array(flags, np.uint32), status=np.array(status, np.uint32))
        print(f"seq_corpus/{name}.npz: {TRIALS} trials, {sum(refused)} refused by the model")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from refpath import require_reference
    main(require_reference(sys.argv))
