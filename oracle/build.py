"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/pcp_oracle.c into oracle/_build/liboracle.so with
-ffp-contract=off so that every FP64 product and sum is rounded as written.
Called by __graft_entry__.build(); safe to call repeatedly (it rebuilds only
when the source is newer than the library).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pcp_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "pcp_oracle.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC",
           "-shared", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
