"""Where the reference tree is, for the tests and fixture generators that
read it (none of the GPU tests do): the CFT_REFERENCE environment variable,
else the location the oracle's build recipe (oracle/Makefile, `refdir`)
knows. None when the tree is absent, as on a GPU host."""
import os
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def reference_root():
    env = os.environ.get("CFT_REFERENCE")
    if env:
        p = Path(env)
        return p if (p / "host" / "src" / "softfloat.c").exists() else None
    try:
        out = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "refdir"],
                             capture_output=True, text=True, timeout=30).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return None
    return Path(out) if out else None


def require_reference(argv):
    """The generators' reference path: argv[1], else reference_root();
    an error when neither names a reference tree."""
    if len(argv) > 1:
        return argv[1]
    r = reference_root()
    if r is None:
        raise SystemExit("the reference tree is needed: pass its path or set CFT_REFERENCE")
    return str(r)
