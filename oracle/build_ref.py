"""Build recipe for oracle/_ref: the reference's own demag code, compiled here.

    python oracle/build_ref.py [--force]

TEST INFRASTRUCTURE ONLY.  Compiles oracle/ref_shim.cpp, which includes the
reference's unmodified src/demag_cu.cu (and through it src/demag_cu.h and
src/constant.h) read in place from the reference checkout, with g++ and the
stand-in headers of oracle/ref_stubs/ (CUDA runtime names as host code,
helper_cuda.h's checkCudaErrors, boost::progress_display).  Two libraries:

    oracle/_ref/libref_demag.so      FLOAT2 = float2  (the reference's default)
    oracle/_ref/libref_demag_f64.so  FLOAT2 = double2 (USE_DOULBE_IN_GPU)

Only the files that compile on their own are used: ktensorCPU, f, g and
calHexchangeKernel.  The rest of the reference (main.cu, the Metropolis,
energy and GPU tensor kernels) cannot be built: their bodies are not
published, and main.cu needs Boost and the CUDA samples' helpers.

The reference checkout exists only on the build machine, so these libraries
are built there, used to generate tests/golden/ref_demag_golden.npz
(tests/golden/make_ref_golden.py) and by the CPU tests when present; nothing
else needs them.  `-ffp-contract=off` keeps the arithmetic as written, like
the oracle's own build.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("MMC_REFERENCE_SRC", "/root/reference/src")
OUT_DIR = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim.cpp")
STUBS = os.path.join(HERE, "ref_stubs")
TARGETS = {
    "libref_demag.so": [],
    "libref_demag_f64.so": ["-DUSE_DOULBE_IN_GPU"],
}


def available():
    """True when the reference sources are present on this machine."""
    return os.path.isfile(os.path.join(REF_SRC, "demag_cu.cu"))


def lib_path(name="libref_demag.so"):
    return os.path.join(OUT_DIR, name)


def _digest():
    h = hashlib.sha256()
    files = [SHIM, __file__] + [os.path.join(REF_SRC, f) for f in ("demag_cu.cu", "demag_cu.h", "constant.h")]
    for root, _, names in os.walk(STUBS):
        files += [os.path.join(root, n) for n in sorted(names)]
    for p in files:
        h.update(p.encode())
        h.update(open(p, "rb").read())
    return h.hexdigest()


def build(force=False):
    """Compile both libraries when the reference sources are present; returns
    the output folder, or None when they are absent."""
    if not available():
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    digest = _digest()
    stamp = os.path.join(OUT_DIR, "stamp")
    if (not force and os.path.exists(stamp) and open(stamp).read() == digest
            and all(os.path.exists(lib_path(t)) for t in TARGETS)):
        return OUT_DIR
    for name, extra in TARGETS.items():
        tmp = lib_path(name) + ".tmp"
        cmd = (["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                "-I" + STUBS, "-I" + REF_SRC] + extra + [SHIM, "-o", tmp])
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
        os.replace(tmp, lib_path(name))
    with open(stamp, "w") as f:
        f.write(digest)
    return OUT_DIR


if __name__ == "__main__":
    out = build(force="--force" in sys.argv)
    print(out if out else "reference sources absent: nothing built")
