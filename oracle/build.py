"""Build recipe for the CPU oracle (test infrastructure only).

    python oracle/build.py

Compiles oracle.cpp into oracle/_build/liboracle.so with -ffp-contract=off so
that its FP64 arithmetic rounds exactly as written, and with OpenMP when the
compiler supports it.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")
DEPS = [SRC, os.path.join(ROOT, "include", "mmc.h"),
        os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300", "csrc", "mmc_math.h")]
BASE = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", SRC]


def build(force=False):
    h = hashlib.sha256()
    for d in DEPS:
        h.update(open(d, "rb").read())
    h.update(open(__file__, "rb").read())
    digest = h.hexdigest()
    stamp = OUT + ".stamp"
    if not force and os.path.exists(OUT) and os.path.exists(stamp) and open(stamp).read() == digest:
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    r = subprocess.run(BASE + ["-fopenmp", "-o", tmp], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:  # no OpenMP runtime: build single-threaded
        r = subprocess.run(BASE + ["-o", tmp], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
    os.replace(tmp, OUT)
    with open(stamp, "w") as f:
        f.write(digest)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
