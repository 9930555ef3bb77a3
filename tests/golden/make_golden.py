"""Generates the golden fixtures in this folder.

    python tests/golden/make_golden.py

newell_golden.json -- the reference's Newell potentials f, g (src/demag_cu.h:43-71,
    with its EPSILON = 1e-200 guards, src/constant.h:23) and the full periodic-image
    tensor sum of ktensorCPU (src/demag_cu.cu:119-248) evaluated with mpmath at 60
    significant digits for a few small lattices.  This is an independent
    high-precision evaluation of the reference's own formulas; it needs mpmath
    (bundled with sympy) and runs in about a minute.
newell_far_golden.json -- the six raw 64-term sums of single image offsets from
    12 to 400 cells away, at 60 digits: the target of the far-field expansion
    (csrc/newell_far.h), which FP64 evaluations of the sums cannot reach there.
    `python tests/golden/make_golden.py --far` writes only this file.
trajectory_fp64.npz -- a short FP64 Metropolis trajectory produced by the CPU
    oracle (oracle/oracle.cpp) on an 8x8x1 periodic film with demag: initial m,
    tensor, demag field, energies and m after 20 sweeps.  A regression pin for the
    oracle and a fixture the GPU tests compare against without running the oracle.
"""
import json
import os
import sys

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

mp.mp.dps = 60
EPS = mp.mpf("1e-200")


def f(x, y, z):
    x, y, z = abs(x), abs(y), abs(z)
    R = mp.sqrt(x * x + y * y + z * z)
    return (y / 2 * (z * z - x * x) * mp.asinh(y / (mp.sqrt(x * x + z * z) + EPS))
            + z / 2 * (y * y - x * x) * mp.asinh(z / (mp.sqrt(x * x + y * y) + EPS))
            - x * y * z * mp.atan(y * z / (x * R + EPS))
            + mp.mpf(1) / 6 * (2 * x * x - y * y - z * z) * R)


def g(x, y, z):
    z = abs(z)
    R = mp.sqrt(x * x + y * y + z * z)
    return (x * y * z * mp.asinh(z / (mp.sqrt(x * x + y * y) + EPS))
            + y / 6 * (3 * z * z - y * y) * mp.asinh(x / (mp.sqrt(y * y + z * z) + EPS))
            + x / 6 * (3 * z * z - x * x) * mp.asinh(y / (mp.sqrt(x * x + z * z) + EPS))
            - z * z * z / 6 * mp.atan(x * y / (z * R + EPS))
            - z * y * y / 2 * mp.atan(x * z / (y * R + EPS))
            - z * x * x / 2 * mp.atan(y * z / (x * R + EPS))
            - x * y * R / 3)


def wrap(x, n):
    return (x + (n + 1) // 2 - 1) % n - (n + 1) // 2 + 1


def tensor(nx, ny, nz, dx, dy, dz, pbc):
    pad = [2 * n - 1 if p == 0 else n for n, p in zip((nx, ny, nz), pbc)]
    P = [max(p, 0) for p in pbc]
    dxm, dym, dzm = mp.mpf(dx), mp.mpf(dy), mp.mpf(dz)
    # f/g on every node the stencils touch, evaluated once
    cache = {}

    def val(fn, key, a, b, c):
        k = (fn, key)
        if k not in cache:
            cache[k] = (f if fn == "f" else g)(a, b, c)
        return cache[k]

    out = np.zeros((6, pad[0] * pad[1] * pad[2]))
    for z in range(pad[2]):
        for y in range(pad[1]):
            for x in range(pad[0]):
                ix0, iy0, iz0 = wrap(x, pad[0]), wrap(y, pad[1]), wrap(z, pad[2])
                acc = [mp.mpf(0)] * 6
                for px in range(-P[0], P[0] + 1):
                    for py in range(-P[1], P[1] + 1):
                        for pz in range(-P[2], P[2] + 1):
                            ix, iy, iz = ix0 + px * pad[0], iy0 + py * pad[1], iz0 + pz * pad[2]
                            for bits in range(64):
                                ikx, iky, ikz = (bits >> 5) & 1, (bits >> 4) & 1, (bits >> 3) & 1
                                ilx, ily, ilz = (bits >> 2) & 1, (bits >> 1) & 1, bits & 1
                                a, b, c = ix + ikx - ilx, iy + iky - ily, iz + ikz - ilz
                                s = 1 if (ikx + iky + ikz + ilx + ily + ilz) % 2 == 0 else -1
                                X, Y, Z = a * dxm, b * dym, c * dzm
                                acc[0] += s * val("f", (a, b, c, 0), X, Y, Z)
                                acc[1] += s * val("g", (a, b, c, 0), X, Y, Z)
                                acc[2] += s * val("g", (a, c, b, 1), X, Z, Y)
                                acc[3] += s * val("f", (b, c, a, 1), Y, Z, X)
                                acc[4] += s * val("g", (b, c, a, 2), Y, Z, X)
                                acc[5] += s * val("f", (c, a, b, 2), Z, X, Y)
                d = -4 * mp.pi * dxm * dym * dzm
                i = x + pad[0] * (y + pad[1] * z)
                for q in range(6):
                    out[q, i] = float(acc[q] / d)
    return pad, out


def raw_sums(ix, iy, iz, dx, dy, dz):
    """The six 64-term sums (xx, xy, xz, yy, yz, zz) of one offset in cells."""
    h = [mp.mpf(dx), mp.mpf(dy), mp.mpf(dz)]
    acc = [mp.mpf(0)] * 6
    for bits in range(64):
        ikx, iky, ikz = (bits >> 5) & 1, (bits >> 4) & 1, (bits >> 3) & 1
        ilx, ily, ilz = (bits >> 2) & 1, (bits >> 1) & 1, bits & 1
        s = 1 if (ikx + iky + ikz + ilx + ily + ilz) % 2 == 0 else -1
        X, Y, Z = (ix + ikx - ilx) * h[0], (iy + iky - ily) * h[1], (iz + ikz - ilz) * h[2]
        acc[0] += s * f(X, Y, Z)
        acc[1] += s * g(X, Y, Z)
        acc[2] += s * g(X, Z, Y)
        acc[3] += s * f(Y, Z, X)
        acc[4] += s * g(Y, Z, X)
        acc[5] += s * f(Z, X, Y)
    return [float(a) for a in acc]


def far_cases():
    cases = []
    for (ix, iy, iz, dx, dy, dz) in [
        (12, 5, 2, 1e-9, 1e-9, 0.8e-9), (20, 7, 3, 1e-9, 1e-9, 0.8e-9), (30, -11, 4, 1e-9, 1e-9, 0.8e-9),
        (-25, 18, 0, 1e-9, 1e-9, 0.8e-9), (0, 40, -3, 2e-9, 2e-9, 1e-9), (64, 0, 0, 1e-9, 1e-9, 0.8e-9),
        (0, 0, 48, 1e-9, 1e-9, 1e-9), (80, -30, 12, 1e-9, 1e-9, 0.8e-9), (-128, 96, 5, 2e-9, 2e-9, 1e-9),
        (256, 0, 0, 1e-9, 1e-9, 0.8e-9), (300, 250, 0, 1e-9, 1e-9, 0.8e-9), (17, 33, 9, 1e-9, 1.5e-9, 1e-9),
    ]:
        cases.append({"cell": [ix, iy, iz], "d": [dx, dy, dz], "raw": raw_sums(ix, iy, iz, dx, dy, dz)})
    with open(os.path.join(HERE, "newell_far_golden.json"), "w") as fh:
        json.dump({"digits": mp.mp.dps, "cases": cases}, fh)


def main():
    far_cases()
    if "--far" in sys.argv:
        return
    rng = np.random.default_rng(2024)
    pts = []
    for _ in range(40):
        v = rng.integers(-6, 7, size=3) * np.array([1e-9, 1e-9, 0.8e-9])
        pts.append([float(t) for t in v])
    pts += [[0.0, 0.0, 0.0], [1e-9, 0.0, 0.0], [0.0, 1e-9, 0.0], [0.0, 0.0, 1e-9], [2e-9, 3e-9, 0.0]]
    fg = [{"x": p, "f": float(f(*map(mp.mpf, p))), "g": float(g(*map(mp.mpf, p)))} for p in pts]
    cases = []
    for (nx, ny, nz, dx, dy, dz, pbc) in [
        (3, 2, 2, 1e-9, 1e-9, 1e-9, (0, 0, 0)),
        (4, 4, 1, 1e-9, 1e-9, 0.8e-9, (1, 1, 0)),
        (3, 2, 1, 2e-9, 1e-9, 1e-9, (-1, 2, 0)),
        (2, 2, 3, 1e-9, 1.5e-9, 1e-9, (0, 1, 0)),
    ]:
        pad, k = tensor(nx, ny, nz, dx, dy, dz, pbc)
        cases.append({"nx": nx, "ny": ny, "nz": nz, "dx": dx, "dy": dy, "dz": dz, "pbc": list(pbc),
                      "padded": pad, "K": k.tolist()})
        print("tensor", nx, ny, nz, pbc, "done", flush=True)
    with open(os.path.join(HERE, "newell_golden.json"), "w") as fh:
        json.dump({"digits": mp.mp.dps, "fg": fg, "tensors": cases}, fh)

    import mmc_ctypes as M
    import oracle_ctypes as O
    cfg = M.Config.defaults(nx=8, ny=8, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=64, randomseed=256,
                            cal_demag_flag=1, tensor_sum=0)
    k6 = O.tensor(cfg)
    m0 = O.init_random(cfg, 256)
    h0 = O.demag_direct(cfg, k6, m0)
    e0 = O.energy(cfg, m0, h0)
    m = m0.copy()
    acc = O.sweeps(cfg, k6, 300.0, 3, 0, 20, m, demag_mode=0)
    h1 = O.demag_direct(cfg, k6, m)
    e1 = O.energy(cfg, m, h1)
    np.savez(os.path.join(HERE, "trajectory_fp64.npz"), k6=k6, m0=m0, h0=h0, e0=e0, m20=m, h20=h1, e20=e1,
             accepted=np.array([acc]), T=np.array([300.0]), stage=np.array([3]), seed=np.array([256]))
    print("trajectory accepted", acc)


if __name__ == "__main__":
    main()
