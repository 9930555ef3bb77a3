"""Build recipe for libmmc.so (sm_103a) and the `mmc` command-line driver.

Translation units are compiled in parallel; an unchanged source tree is not
rebuilt.  FP64 kernels are compiled with -fmad=false and host code with
-ffp-contract=off so that FP64 results round the same way as the CPU oracle.

    python build.py            # build if needed
    python build.py --force    # rebuild everything
"""
import argparse
import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libmmc.so")
CLI = os.path.join(BINDIR, "mmc")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I" + os.path.join(ROOT, "include")]
GXX_COMMON = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
              "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA_HOME, "include")]

# (source, extra flags, compiler)
UNITS = [
    ("kernels_f32.cu", ["-fmad=true"], "nvcc"),
    ("kernels_f64.cu", ["-fmad=false"], "nvcc"),
    ("newell.cu", ["-fmad=false"], "nvcc"),
    ("demag_static.cu", [], "nvcc"),
    ("runtime.cpp", [], "g++"),
    ("ini.cpp", [], "g++"),
    ("ovf.cpp", [], "g++"),
]


def _tree_hash():
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include"), os.path.join(HERE, "cli")):
        for name in sorted(os.listdir(d)):
            p = os.path.join(d, name)
            if os.path.isfile(p):
                h.update(name.encode())
                with open(p, "rb") as f:
                    h.update(f.read())
    h.update(repr((UNITS, NVCC_COMMON, GXX_COMMON)).encode())
    h.update(open(__file__, "rb").read())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _compile(unit):
    src, extra, comp = unit
    obj = os.path.join(BUILD, src + ".o")
    if comp == "nvcc":
        cmd = [NVCC] + NVCC_COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    else:
        cmd = GXX_COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    _run(cmd)
    return obj


def build(force=False, verbose=False):
    """Compile libmmc.so and bin/mmc; returns the library path."""
    stamp = os.path.join(BUILD, "stamp")
    digest = _tree_hash()
    if not force and os.path.exists(LIB) and os.path.exists(CLI) and os.path.exists(stamp):
        if open(stamp).read().strip() == digest:
            return LIB
    for d in (BUILD, LIBDIR, BINDIR):
        os.makedirs(d, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    os.replace(tmp, LIB)
    _run(GXX_COMMON + [os.path.join(HERE, "cli", "mmc_main.cpp"), "-o", CLI, "-L" + LIBDIR, "-lmmc",
                       "-Wl,-rpath,$ORIGIN/../lib"])
    with open(stamp, "w") as f:
        f.write(digest)
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


def clean():
    for d in (BUILD, LIBDIR, BINDIR):
        shutil.rmtree(d, ignore_errors=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--clean", action="store_true")
    a = ap.parse_args()
    if a.clean:
        clean()
        sys.exit(0)
    build(force=a.force, verbose=True)
