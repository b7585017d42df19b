"""The serving loop's budget allocator (csrc/arena.h), compiled on its own
with the host C++ compiler and driven with random traffic."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_arena_random_traffic(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "arena_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "cft-fp256_gb300" / "csrc"),
                    str(ROOT / "tests" / "arena_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
