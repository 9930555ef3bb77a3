"""ctypes wrapper of the CPU oracle (oracle.cpp).  TEST INFRASTRUCTURE ONLY:
imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.

Arrays are numpy float64, SoA: m has shape (3, n), n = nx*ny*nz, x fastest.
"""
import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300")


def _load_module(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_build = _load_module("oracle_build", os.path.join(HERE, "build.py"))

_LIB = None
# "shared": liboracle.so (the product's elementary functions, for bit-level
# comparison with the GPU); "libm": liboracle_libm.so (see independent()).
_VARIANT = "shared"
_INDEP = None
_dp = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)


def _config_type():
    import sys
    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    import mmc_ctypes
    return mmc_ctypes.Config


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build(variant=_VARIANT)
    L = ctypes.CDLL(path)
    C = ctypes.c_void_p  # pointer to mmc_config
    sig = {
        "orc_padded_dims": (ctypes.c_int, [C, ctypes.POINTER(ctypes.c_int)]),
        "orc_newell_f": (ctypes.c_double, [ctypes.c_double] * 3),
        "orc_newell_g": (ctypes.c_double, [ctypes.c_double] * 3),
        "orc_math": (None, [ctypes.c_int, _dp, _dp, ctypes.c_long]),
        "orc_philox": (None, [_u32p, _u32p, _u32p]),
        "orc_newell_tensor": (ctypes.c_int, [C, _dp]),
        "orc_init_random": (None, [C, ctypes.c_longlong, _dp]),
        "orc_demag_direct": (ctypes.c_int, [C, _dp, _dp, _dp]),
        "orc_demag_fft": (ctypes.c_int, [C, _dp, _dp, _dp]),
        "orc_field": (ctypes.c_int, [C, ctypes.c_int, _dp, _dp, _dp]),
        "orc_energy": (ctypes.c_int, [C, _dp, _dp, _dp]),
        "orc_grad": (ctypes.c_int, [C, _dp, _dp, _dp, _dp]),
        "orc_newell_far": (None, [ctypes.c_double] * 6 + [_dp]),
        "orc_newell_raw": (None, [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [_dp]),
        "orc_sweeps": (ctypes.c_int, [C, _dp, ctypes.c_double, ctypes.c_longlong, ctypes.c_longlong,
                                      ctypes.c_longlong, _dp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int,
                                      ctypes.c_int]),
        "orc_energy_total": (ctypes.c_double, [C, _dp, _dp]),
        "orc_demag_product": (None, [ctypes.c_long, _dp, _dp, _dp]),
        "orc_newell_points": (ctypes.c_int, [C, ctypes.POINTER(ctypes.c_long), ctypes.c_long, _dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def independent():
    """This API bound to liboracle_libm.so: the oracle built with the C
    library's elementary functions and its own Philox, sharing no code with
    the product (no far-field tensor form)."""
    global _INDEP
    if _VARIANT == "libm":
        return sys.modules[__name__]
    if _INDEP is None:
        mod = _load_module("oracle_ctypes_libm", os.path.abspath(__file__))
        mod._VARIANT = "libm"
        sys.modules["oracle_ctypes_libm"] = mod
        _INDEP = mod
    return _INDEP


def config(**kw):
    """An mmc_config for the oracle alone (zero-initialised, then kw), without
    loading the product library: the oracle reads only the geometry, the
    material, the seed, use_reference_pi and tensor_far_radius."""
    c = _config_type()()
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _c(cfg):
    return ctypes.cast(ctypes.byref(cfg), ctypes.c_void_p)


def _p(a):
    return a.ctypes.data_as(_dp)


def padded_dims(cfg):
    out = (ctypes.c_int * 3)()
    lib().orc_padded_dims(_c(cfg), out)
    return tuple(out)


def newell_f(x, y, z):
    return lib().orc_newell_f(x, y, z)


def newell_g(x, y, z):
    return lib().orc_newell_g(x, y, z)


MATH = {"log": 0, "asinh": 1, "atan": 2, "exp": 3, "sinpi": 4, "cospi": 5}


def math(fn, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().orc_math(MATH[fn], _p(x), _p(y), x.size)
    return y


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(c.ctypes.data_as(_u32p), k.ctypes.data_as(_u32p), o.ctypes.data_as(_u32p))
    return o


def tensor(cfg):
    nxp, nyp, nzp = padded_dims(cfg)
    k = np.zeros((6, nxp * nyp * nzp))
    lib().orc_newell_tensor(_c(cfg), _p(k))
    return k


def tensor_points(cfg, idx):
    """The tensor at flat padded-grid indices idx (x fastest): shape (6, len(idx))."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros((6, idx.size))
    rc = lib().orc_newell_points(_c(cfg), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), idx.size, _p(out))
    assert rc == 0, rc
    return out


def demag_product(mhat, khat):
    """H^ = K^ . M^ / N per frequency: mhat complex (3, np), khat complex (6, np)."""
    m = np.ascontiguousarray(mhat, dtype=np.complex128)
    k = np.ascontiguousarray(khat, dtype=np.complex128)
    h = np.zeros_like(m)
    np_ = m.shape[1]
    lib().orc_demag_product(np_, m.ctypes.data_as(_dp), k.ctypes.data_as(_dp), h.ctypes.data_as(_dp))
    return h


def init_random(cfg, seed):
    n = cfg.nx * cfg.ny * cfg.nz
    m = np.zeros((3, n))
    lib().orc_init_random(_c(cfg), seed, _p(m))
    return m


def demag_direct(cfg, k6, m):
    h = np.zeros_like(m, dtype=np.float64)
    lib().orc_demag_direct(_c(cfg), _p(np.ascontiguousarray(k6)), _p(np.ascontiguousarray(m, dtype=np.float64)), _p(h))
    return h


def demag_fft(cfg, k6, m):
    h = np.zeros_like(m, dtype=np.float64)
    lib().orc_demag_fft(_c(cfg), _p(np.ascontiguousarray(k6)), _p(np.ascontiguousarray(m, dtype=np.float64)), _p(h))
    return h


def field(cfg, term, m, hd=None):
    m = np.ascontiguousarray(m, dtype=np.float64)
    H = np.zeros_like(m)
    hp = _p(np.ascontiguousarray(hd, dtype=np.float64)) if hd is not None else None
    lib().orc_field(_c(cfg), term, _p(m), hp, _p(H))
    return H


def energy(cfg, m, hd=None):
    """[E_ex, E_dmi, E_an, E_zeeman, E_demag, <mx>, <my>, <mz>, Q]."""
    m = np.ascontiguousarray(m, dtype=np.float64)
    out = np.zeros(9)
    hp = _p(np.ascontiguousarray(hd, dtype=np.float64)) if hd is not None else None
    lib().orc_energy(_c(cfg), _p(m), hp, _p(out))
    return out


def newell_far(X, Y, Z, dx, dy, dz):
    """Far-field form of the six raw 64-term sums of one offset (metres)."""
    out = np.zeros(6)
    lib().orc_newell_far(X, Y, Z, dx, dy, dz, _p(out))
    return out


def newell_raw(ix, iy, iz, dx, dy, dz):
    """The exact six raw 64-term sums of one offset in cells (FP64)."""
    out = np.zeros(6)
    lib().orc_newell_raw(ix, iy, iz, dx, dy, dz, _p(out))
    return out


def grad(cfg, k6, m):
    """(dE/dm as float64 (3, n), dE/d(Aex, Dind, Ku1, Ms, Bx, By, Bz))."""
    m = np.ascontiguousarray(m, dtype=np.float64)
    g = np.zeros_like(m)
    dp = np.zeros(7)
    kp = _p(np.ascontiguousarray(k6)) if k6 is not None else None
    assert lib().orc_grad(_c(cfg), kp, _p(m), _p(g), _p(dp)) == 0
    return g, dp


def sweeps(cfg, k6, T, stage, sweep0, nsweeps, m, demag_mode=1, nthreads=0):
    """Runs nsweeps sweeps in place on m (float64 (3, n)); returns the accept count."""
    assert m.dtype == np.float64 and m.flags.c_contiguous
    acc = ctypes.c_ulonglong(0)
    kp = _p(np.ascontiguousarray(k6)) if k6 is not None else None
    lib().orc_sweeps(_c(cfg), kp, float(T), stage, sweep0, nsweeps, _p(m), ctypes.byref(acc), demag_mode, nthreads)
    return acc.value
