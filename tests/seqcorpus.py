"""The reference's sequencer differential corpus (host/tests/seq_check.py's
first corpus, with the golden model's results; tests/golden/
make_seq_corpus.py), trial by trial."""
from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden" / "seq_corpus"
NAMES = ("fp32", "fp64", "fp128", "fp256")


def trials(fmt):
    z = np.load(GOLD / f"{NAMES[fmt]}.npz")
    io, do = z["img_off"], z["dep_off"]
    s = c = 0
    for t in range(len(z["refused"])):
        img = z["images"][io[t]:io[t + 1]].copy()
        n = int(z["n"][t])
        tr = dict(trial=t, image=img, refused=bool(z["refused"][t]), n=n)
        if not tr["refused"]:
            st = z["streams"][s:s + 3 * n]
            s += 3 * n
            tr.update(a=st[:n].copy(), b=st[n:2 * n].copy(), c=st[2 * n:].copy(),
                      deposits=z["deposits"][do[t]:do[t + 1]].copy(),
                      counts=z["counts"][c:c + n].copy(), flags=int(z["flags"][t]),
                      status=int(z["status"][t]))
            c += n
        yield tr
