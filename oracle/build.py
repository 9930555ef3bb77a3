"""Build recipe for the CPU oracle (test infrastructure only).

    python oracle/build.py [--force]

Compiles oracle.cpp twice, with -ffp-contract=off so that its FP64
arithmetic rounds exactly as written, and with OpenMP when the compiler
supports it:

    oracle/_build/liboracle.so       elementary functions and Philox from the
                                     product's csrc/mmc_math.h, so that FP64
                                     results compare bit for bit with the GPU
    oracle/_build/liboracle_libm.so  -DORACLE_LIBM: the C library's functions
                                     and the oracle's own Philox; nothing of
                                     the product enters (its tensor equals the
                                     reference's compiled ktensorCPU bit for bit)
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "oracle.cpp")
DEPS = [SRC, os.path.join(ROOT, "include", "mmc.h"),
        os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300", "csrc", "mmc_math.h"),
        os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300", "csrc", "newell_far.h")]
BASE = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", SRC]
VARIANTS = {"shared": ("liboracle.so", []), "libm": ("liboracle_libm.so", ["-DORACLE_LIBM"])}


def out_path(variant="shared"):
    return os.path.join(HERE, "_build", VARIANTS[variant][0])


def _digest(variant):
    h = hashlib.sha256()
    for d in DEPS:
        h.update(open(d, "rb").read())
    h.update(open(__file__, "rb").read())
    h.update(variant.encode())
    return h.hexdigest()


def build(force=False, variant="shared"):
    """Compiles one variant if its sources changed; returns its path."""
    out = out_path(variant)
    digest = _digest(variant)
    stamp = out + ".stamp"
    if not force and os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == digest:
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp"
    extra = VARIANTS[variant][1]
    r = subprocess.run(BASE + extra + ["-fopenmp", "-o", tmp], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode != 0:  # no OpenMP runtime: build single-threaded
        r = subprocess.run(BASE + extra + ["-o", tmp], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(digest)
    return out


def build_all(force=False):
    return [build(force, v) for v in VARIANTS]


if __name__ == "__main__":
    for p in build_all(force="--force" in sys.argv):
        print(p)
