"""Generates tests/golden/ref_demag_golden.npz from the reference's own code.

    python oracle/build_ref.py && python tests/golden/make_ref_golden.py

Runs only where the reference sources are present (the libraries of
oracle/_ref, built by oracle/build_ref.py from the unmodified
src/demag_cu.cu).  Everything stored is an output of the reference's code:

- K_<case>: ktensorcpu::ktensorCPU (src/demag_cu.cu:119-248) on the padded
  grid of each case, transposed to x fastest; the reference's CONST_PI
  (3.14159265358, src/constant.h:21), so compare with use_reference_pi = 1.
  Cases: the four lattices of newell_golden.json, a 6x5x4 open slab, an 8x8x3
  film with 2 images in x and y, and the 64x64x1 film with 20 images in x and
  y and dx = dy = 1 nm, dz = 0.8 nm (about five minutes of CPU time).
- P_*: calHexchangeKernel (src/demag_cu.cu:68-116) run over its launch grid on
  seeded random spectra of a 5x4x3 grid, in the double2 and float2 builds.
- H64_<case>, H32_<case>: the demag field h = K * m (dimensionless, H = Ms h)
  of m = the seeded initial state (sha256 of its FP64 bytes stored beside it),
  formed the reference's way: forward FFT of the zero-padded m and of the
  reference tensor, the reference's K^.M^/N product, unnormalised inverse FFT
  and crop (the inverse and crop the reference leaves out, src/main.cu:868-900).
  numpy's FFT stands in for cuFFT.  H32 runs the product in the float2 build
  on complex64 spectra (m and K^ rounded to FP32 first, as the reference's
  FP32 build holds them) and the inverse in complex64.

The m of each field case comes from the oracle's seeded initial state, which
the GPU reproduces bit for bit; the tests check the hash before comparing.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mmc_ctypes as M  # noqa: E402  (Config only: no GPU call)
import oracle_ctypes as O  # noqa: E402
import ref_ctypes as R  # noqa: E402

OUT = os.path.join(HERE, "ref_demag_golden.npz")

CASES = {
    "g0_3x2x2_open": dict(nx=3, ny=2, nz=2, dx=1e-9, dy=1e-9, dz=1e-9, pbc=(0, 0, 0)),
    "g1_4x4x1_pbc1": dict(nx=4, ny=4, nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, pbc=(1, 1, 0)),
    "g2_3x2x1_mixed": dict(nx=3, ny=2, nz=1, dx=2e-9, dy=1e-9, dz=1e-9, pbc=(-1, 2, 0)),
    "g3_2x2x3_mixed": dict(nx=2, ny=2, nz=3, dx=1e-9, dy=1.5e-9, dz=1e-9, pbc=(0, 1, 0)),
    "slab6x5x4_open": dict(nx=6, ny=5, nz=4, dx=1e-9, dy=1.2e-9, dz=0.7e-9, pbc=(0, 0, 0)),
    "film8x8x3_pbc2": dict(nx=8, ny=8, nz=3, dx=1e-9, dy=1e-9, dz=1e-9, pbc=(2, 2, 0)),
    "cfg0_64x64x1_pbc20": dict(nx=64, ny=64, nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, pbc=(20, 20, 0)),
}
# demag-field cases: (tensor case, seed of the initial state)
FIELDS = {"slab6x5x4_open": 7, "film8x8x3_pbc2": 11, "cfg0_64x64x1_pbc20": 256}


def config(case):
    c = CASES[case]
    return M.Config.defaults(nx=c["nx"], ny=c["ny"], nz=c["nz"], dx=c["dx"], dy=c["dy"], dz=c["dz"],
                             pbc_x=c["pbc"][0], pbc_y=c["pbc"][1], pbc_z=c["pbc"][2], use_reference_pi=1)


def ref_field(case, k, m, fp64):
    """h = crop(IFFT(K^.M^/N)) with the reference's product (see module doc)."""
    c = CASES[case]
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    dims = R.padded(nx, ny, nz, c["pbc"])
    nxp, nyp, nzp = dims
    # arrays indexed [z, y, x] (x fastest) on the padded grid
    kk = k.reshape(6, nzp, nyp, nxp)
    mp = np.zeros((3, nzp, nyp, nxp))
    mp[:, :nz, :ny, :nx] = m.reshape(3, nz, ny, nx)
    axes = (1, 2, 3)
    khat = np.fft.fftn(kk, axes=axes)  # FP64 (the reference's D2Z of the tensor)
    if fp64:
        mhat = np.fft.fftn(mp, axes=axes)
    else:
        mhat = np.fft.fftn(mp.astype(np.float32), axes=axes)
        khat = khat.astype(np.complex64)
    hhat = R.hexchange(mhat.reshape(3, -1), khat.reshape(6, -1), dims, fp64=fp64).reshape(3, nzp, nyp, nxp)
    h = np.fft.ifftn(hhat, axes=axes, norm="forward").real
    return np.ascontiguousarray(h[:, :nz, :ny, :nx]).reshape(3, -1)


def main():
    assert R.available(), "the reference sources are not on this machine"
    out, meta = {}, {"cases": CASES, "fields": FIELDS, "const_pi": R.lib().ref_const_pi()}
    for name, c in CASES.items():
        t = time.time()
        out["K_" + name] = R.ktensor(c["nx"], c["ny"], c["nz"], c["dx"], c["dy"], c["dz"], c["pbc"])
        print(name, "tensor %.1f s" % (time.time() - t), flush=True)
    rng = np.random.default_rng(2024)
    dims = (5, 4, 3)
    npp = int(np.prod(dims))
    mh = rng.standard_normal((3, npp)) + 1j * rng.standard_normal((3, npp))
    kh = rng.standard_normal((6, npp)) + 1j * rng.standard_normal((6, npp))
    out["P_dims"] = np.array(dims)
    out["P_m"], out["P_k"] = mh, kh
    out["P_h64"] = R.hexchange(mh, kh, dims, fp64=True)
    out["P_h32"] = R.hexchange(mh.astype(np.complex64), kh.astype(np.complex64), dims, fp64=False)
    for name, seed in FIELDS.items():
        cfg = config(name)
        m = O.init_random(cfg, seed)
        meta.setdefault("m_sha256", {})[name] = hashlib.sha256(m.tobytes()).hexdigest()
        k = out["K_" + name]
        out["H64_" + name] = ref_field(name, k, m, True)
        out["H32_" + name] = ref_field(name, k, m, False).astype(np.float32)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
