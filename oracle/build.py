"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/rast_oracle.c into oracle/_build/liboracle.so with IEEE single-precision
semantics: -ffp-contract=off (GCC on aarch64 fuses a*b+c into fmadd by default, which would
break bit-exactness with the reference's release build) and no -ffast-math.

The reference crate itself (Rust) cannot be built on these machines (no rustc/cargo), so
there is no oracle/_ref build; the restatement is pinned by the reference's unit tests.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "rast_oracle.c")]
HDR = [os.path.join(HERE, "rast_oracle.h")]

CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-pthread", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + HDR + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc"] + CFLAGS + SRC + ["-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
