"""Build recipe for the oracle (test infrastructure, not product code).

Compiles oracle/lbm_oracle.c (with the .inc files it includes) into oracle/_build/liblbm_oracle.so with OpenMP and with
floating-point contraction disabled, so that every float operation of the restatement
rounds exactly where the WGSL expression it follows rounds.  No architecture-specific
flags: the same source builds on the x86_64 build host and on the aarch64 GPU host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblbm_oracle.so")
SOURCES = ["lbm_oracle.c"]
DEPS = SOURCES + ["lbm_oracle.h", "lbm_oracle_phys.inc", "lbm_oracle_view.inc"]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, d)) > t for d in DEPS)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-std=c11", "-Wall", "-o", tmp] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
