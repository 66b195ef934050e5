"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/sf_oracle.c`` with gcc into ``oracle/_build/libsf_oracle.so``.
Portable C: the NEON row kernel is compiled only on aarch64 hosts, scalar
rows elsewhere; no host-specific flags.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sf_oracle.c")
HDR = os.path.join(HERE, "sf_oracle.h")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsf_oracle.so")


def command(out: str = LIB) -> list[str]:
    return ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-Wall",
            "-Wno-unused-function", SRC, "-o", out]


def stale(out: str = LIB) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(f) > t for f in (SRC, HDR, __file__))


def start(out: str = LIB) -> subprocess.Popen | None:
    """Start the compile (None when the library is up to date)."""
    if not stale(out):
        return None
    os.makedirs(os.path.dirname(out), exist_ok=True)
    return subprocess.Popen(command(out + ".tmp"), stdout=subprocess.PIPE,
                            stderr=subprocess.STDOUT, text=True)


def finish(proc: subprocess.Popen | None, out: str = LIB) -> None:
    if proc is None:
        return
    log, _ = proc.communicate()
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + log)
    os.replace(out + ".tmp", out)


def build(out: str = LIB) -> str:
    finish(start(out), out)
    return out


if __name__ == "__main__":
    print(build())
    sys.exit(0)
