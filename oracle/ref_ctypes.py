"""ctypes wrapper of oracle/_ref: the reference's own demag code compiled here
(oracle/build_ref.py).  TEST INFRASTRUCTURE ONLY: used by
tests/golden/make_ref_golden.py and by the CPU tests on a machine that holds
the reference sources; elsewhere available() is False and those tests use the
committed fixtures instead.

Arrays follow the oracle's conventions: tensors (6, np) with x fastest, so the
reference's z-fastest layout (src/demag_cu.cu:146) is transposed here.
"""
import ctypes
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_module(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_build = _load_module("ref_build", os.path.join(HERE, "build_ref.py"))
_LIBS = {}
_dp = ctypes.POINTER(ctypes.c_double)


def available():
    return _build.available()


def lib(fp64=True):
    """libref_demag_f64.so (FLOAT2 = double2) or libref_demag.so (float2)."""
    name = "libref_demag_f64.so" if fp64 else "libref_demag.so"
    if name in _LIBS:
        return _LIBS[name]
    if _build.build() is None:
        raise RuntimeError("the reference sources are not on this machine")
    L = ctypes.CDLL(_build.lib_path(name))
    for fn in ("ref_f_host", "ref_g_host", "ref_f_devsrc", "ref_g_devsrc"):
        getattr(L, fn).restype = ctypes.c_double
        getattr(L, fn).argtypes = [ctypes.c_double] * 3
    L.ref_const_pi.restype = ctypes.c_double
    L.ref_float2_bytes.restype = ctypes.c_int
    L.ref_ktensor.restype = ctypes.c_long
    L.ref_ktensor.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [ctypes.c_int] * 3 + [_dp]
    L.ref_hexchange.restype = None
    L.ref_hexchange.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 3
    _LIBS[name] = L
    return L


def fg(name, pts):
    """One of ref_f_host, ref_g_host, ref_f_devsrc, ref_g_devsrc over rows of pts (k, 3)."""
    fn = getattr(lib(), name)
    return np.array([fn(float(a), float(b), float(c)) for a, b, c in np.asarray(pts, dtype=np.float64)])


def padded(nx, ny, nz, pbc):
    """src/main.cu:254-260: an open axis (pbc == 0) pads n to 2n - 1."""
    return tuple(2 * n - 1 if p == 0 else n for n, p in zip((nx, ny, nz), pbc))


def ktensor(nx, ny, nz, dx, dy, dz, pbc):
    """ktensorCPU on the padded grid of (nx, ny, nz), images max(pbc, 0) per
    axis (src/main.cu:537-539 turns pbc < 0 into no images); shape (6, np)
    with x fastest."""
    nxp, nyp, nzp = padded(nx, ny, nz, pbc)
    k = np.zeros((6, nxp, nyp, nzp))
    P = [max(int(p), 0) for p in pbc]
    n = lib().ref_ktensor(nxp, nyp, nzp, dx, dy, dz, P[0], P[1], P[2], k.ctypes.data_as(_dp))
    assert n == nxp * nyp * nzp
    return np.ascontiguousarray(k.transpose(0, 3, 2, 1)).reshape(6, -1)


def hexchange(mhat, khat, dims, fp64=True):
    """calHexchangeKernel on flat spectra: mhat (3, np), khat (6, np) complex;
    dims = the padded (nxp, nyp, nzp) that set the kernel's grid and its N.
    fp64 selects the double2 build, else the float2 (complex64) one."""
    dt = np.complex128 if fp64 else np.complex64
    m = np.ascontiguousarray(mhat, dtype=dt)
    k = np.ascontiguousarray(khat, dtype=dt)
    assert m.shape[1] == int(np.prod(dims)) and k.shape == (6, m.shape[1])
    h = np.zeros_like(m)
    L = lib(fp64)
    assert L.ref_float2_bytes() == np.dtype(dt).itemsize
    L.ref_hexchange(int(dims[0]), int(dims[1]), int(dims[2]), m.ctypes.data, k.ctypes.data, h.ctypes.data)
    return h
