"""ctypes binding of libmmc (include/mmc.h) used by the Python test harness and
by bench.py.  The product itself is the C ABI; this module only marshals
numpy arrays across it.

    import mmc_ctypes as M
    cfg = M.Config.defaults(nx=64, ny=64)
    with M.Lattice(cfg) as lat:
        lat.run_sweeps(300.0, stage=0, sweep0=0, nsweeps=100)
        obs = lat.energy()
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", "libmmc.so")
HEADER = os.path.join(ROOT, "include", "mmc.h")

OK = 0
ERR_INVALID, ERR_CONFIG, ERR_IO, ERR_CUDA, ERR_NO_DEVICE = 1, 2, 3, 4, 5
ERR_UNSUPPORTED, ERR_INTERRUPTED, ERR_TIMEOUT, ERR_STATE, ERR_OOM = 6, 7, 8, 9, 10
TERM_EXCHANGE, TERM_DMI, TERM_ANISOTROPY, TERM_ZEEMAN, TERM_DEMAG, TERM_TOTAL = range(6)
OVF_BINARY4, OVF_BINARY8, OVF_TEXT = 0, 1, 2
ENGINE_AUTO, ENGINE_KERNELS, ENGINE_FUSED = 0, 1, 2


class Config(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("Bextx", ctypes.c_double), ("Bexty", ctypes.c_double), ("Bextz", ctypes.c_double),
        ("pbc_x", ctypes.c_int), ("pbc_y", ctypes.c_int), ("pbc_z", ctypes.c_int),
        ("ms", ctypes.c_double), ("Aex", ctypes.c_double), ("Dind", ctypes.c_double),
        ("anisUx", ctypes.c_double), ("anisUy", ctypes.c_double), ("anisUz", ctypes.c_double),
        ("Ku1", ctypes.c_double),
        ("use_random_init", ctypes.c_int),
        ("randomseed", ctypes.c_longlong),
        ("ovf_filename", ctypes.c_char * 1024),
        ("Temperature_start", ctypes.c_double), ("Temperature_end", ctypes.c_double),
        ("Temperature_step", ctypes.c_double),
        ("circle_per_stage", ctypes.c_longlong),
        ("terminal_output_period", ctypes.c_longlong),
        ("energy_output_period", ctypes.c_longlong),
        ("ms_output_period", ctypes.c_longlong),
        ("rand_block_size", ctypes.c_int),
        ("cal_demag_flag", ctypes.c_int),
        ("Temperature_use_exp", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("ovf_format", ctypes.c_int),
        ("use_reference_pi", ctypes.c_int),
        ("tensor_cache", ctypes.c_char * 1024),
        ("sweep_engine", ctypes.c_int),
        ("fused_band", ctypes.c_int),
        ("tensor_far_radius", ctypes.c_int),
        ("debug_h_field", ctypes.c_int),
        ("tensor_sum", ctypes.c_int),
    ]

    @classmethod
    def defaults(cls, **kw):
        c = cls()
        lib().mmc_config_defaults(ctypes.byref(c))
        for k, v in kw.items():
            if k in ("ovf_filename", "tensor_cache") and isinstance(v, str):
                v = v.encode()
            setattr(c, k, v)
        return c

    def copy(self, **kw):
        c = Config()
        ctypes.pointer(c)[0] = self
        for k, v in kw.items():
            if k in ("ovf_filename", "tensor_cache") and isinstance(v, str):
                v = v.encode()
            setattr(c, k, v)
        return c


class Observables(ctypes.Structure):
    _fields_ = [
        ("e_total", ctypes.c_double), ("e_exchange", ctypes.c_double), ("e_dmi", ctypes.c_double),
        ("e_anisotropy", ctypes.c_double), ("e_zeeman", ctypes.c_double), ("e_demag", ctypes.c_double),
        ("m", ctypes.c_double * 3), ("q", ctypes.c_double),
        ("accepted", ctypes.c_ulonglong), ("proposed", ctypes.c_ulonglong),
    ]

    def as_dict(self):
        return {
            "e_total": self.e_total, "e_exchange": self.e_exchange, "e_dmi": self.e_dmi,
            "e_anisotropy": self.e_anisotropy, "e_zeeman": self.e_zeeman, "e_demag": self.e_demag,
            "m": list(self.m), "q": self.q, "accepted": self.accepted, "proposed": self.proposed,
        }


class MmcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"mmc status {status}: {msg}")
        self.status = status


_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)


def lib(path=None):
    """Loads libmmc.so once (building it first if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location("mmc_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = ctypes.CDLL(path)
    H = ctypes.c_void_p
    sig = {
        "mmc_abi_version": (ctypes.c_int, []),
        "mmc_config_size": (ctypes.c_size_t, []),
        "mmc_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "mmc_last_error": (ctypes.c_char_p, []),
        "mmc_config_defaults": (None, [ctypes.POINTER(Config)]),
        "mmc_config_load_ini": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Config)]),
        "mmc_config_format": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p, ctypes.c_size_t]),
        "mmc_padded_dims": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_int)]),
        "mmc_transform_dims": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_int)]),
        "mmc_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_int, ctypes.POINTER(H)]),
        "mmc_destroy": (None, [H]),
        "mmc_init_random": (ctypes.c_int, [H, ctypes.c_longlong]),
        "mmc_set_m": (ctypes.c_int, [H, _dp, _dp, _dp]),
        "mmc_get_m": (ctypes.c_int, [H, _dp, _dp, _dp]),
        "mmc_build_demag": (ctypes.c_int, [H, ctypes.c_char_p]),
        "mmc_get_tensor": (ctypes.c_int, [H, _dp]),
        "mmc_self_tensor": (ctypes.c_int, [H, _dp]),
        "mmc_compute_demag": (ctypes.c_int, [H]),
        "mmc_demag_scratch_bytes": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_size_t)]),
        "mmc_demag_apply": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                           ctypes.c_void_p]),
        "mmc_demag_apply_static": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
        "mmc_grad": (ctypes.c_int, [H, _dp, _dp]),
        "mmc_relax": (ctypes.c_int, [H, ctypes.c_double, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong),
                                     _dp]),
        "mmc_get_field": (ctypes.c_int, [H, ctypes.c_int, _dp, _dp, _dp]),
        "mmc_energy": (ctypes.c_int, [H, ctypes.POINTER(Observables)]),
        "mmc_run_sweeps": (ctypes.c_int, [H, ctypes.c_double, ctypes.c_longlong, ctypes.c_longlong,
                                          ctypes.c_longlong]),
        "mmc_run_anneal": (ctypes.c_int, [H, ctypes.c_char_p, ctypes.c_int]),
        "mmc_request_stop": (None, [H]),
        "mmc_last_run_ms": (ctypes.c_int, [H, _dp]),
        "mmc_engine_info": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int)]),
        "mmc_profile_fused": (ctypes.c_int, [H, ctypes.c_double, ctypes.c_longlong, ctypes.c_longlong,
                                             ctypes.c_longlong, ctypes.POINTER(ctypes.c_ulonglong)]),
        "mmc_profile_sweeps": (ctypes.c_int, [H, ctypes.c_double, ctypes.c_longlong, ctypes.c_longlong,
                                              ctypes.c_longlong, _dp]),
        "mmc_ovf_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]),
        "mmc_ovf_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, ctypes.c_int,
                                         ctypes.c_char_p]),
        "mmc_batch_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_int, ctypes.c_int, ctypes.POINTER(H)]),
        "mmc_batch_destroy": (None, [H]),
        "mmc_batch_size": (ctypes.c_int, [H]),
        "mmc_batch_build_demag": (ctypes.c_int, [H, ctypes.c_char_p]),
        "mmc_batch_set_temperatures": (ctypes.c_int, [H, _dp]),
        "mmc_batch_get_temperatures": (ctypes.c_int, [H, _dp]),
        "mmc_batch_set_ladders": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp,
                                                 ctypes.c_int, ctypes.c_longlong]),
        "mmc_batch_ladder_state": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_ulonglong)]),
        "mmc_batch_run_sweeps": (ctypes.c_int, [H, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong]),
        "mmc_batch_last_run_ms": (ctypes.c_int, [H, _dp]),
        "mmc_batch_profile_sweeps": (ctypes.c_int, [H, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                                    _dp]),
        "mmc_batch_launch_shape": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int)]),
        "mmc_batch_autotune": (ctypes.c_int, [H, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int)]),
        "mmc_batch_set_launch_shape": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int)]),
        "mmc_farm_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
        "mmc_farm_destroy": (None, [H]),
        "mmc_farm_run_sweeps": (ctypes.c_int, [H, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong]),
        "mmc_farm_last_run_ms": (ctypes.c_int, [H, _dp]),
        "mmc_farm_request_stop": (None, [H]),
        "mmc_selftest_barrier_timeout": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong,
                                                        ctypes.POINTER(ctypes.c_int)]),
        "mmc_selftest_mbar_timeout": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong,
                                                     ctypes.POINTER(ctypes.c_int)]),
        "mmc_set_stream": (ctypes.c_int, [H, ctypes.c_void_p]),
        "mmc_batch_set_stream": (ctypes.c_int, [H, ctypes.c_void_p]),
        "mmc_batch_request_stop": (None, [H]),
        "mmc_batch_energy": (ctypes.c_int, [H, ctypes.POINTER(Observables)]),
        "mmc_batch_set_m": (ctypes.c_int, [H, ctypes.c_int, _dp, _dp, _dp]),
        "mmc_batch_get_m": (ctypes.c_int, [H, ctypes.c_int, _dp, _dp, _dp]),
        "mmc_selftest_philox": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong, _u32p, ctypes.c_uint32,
                                               ctypes.c_uint32, _u32p, _u32p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if L.mmc_config_size() != ctypes.sizeof(Config):
        raise RuntimeError("mmc_config layout mismatch: library %d bytes, binding %d bytes"
                           % (L.mmc_config_size(), ctypes.sizeof(Config)))
    _LIB = L
    return L


def check(status):
    if status != OK:
        msg = lib().mmc_last_error().decode(errors="replace")
        raise MmcError(status, msg)


def dptr(a):
    return a.ctypes.data_as(_dp)


def load_ini(path):
    c = Config()
    check(lib().mmc_config_load_ini(str(path).encode(), ctypes.byref(c)))
    return c


def format_config(cfg):
    buf = ctypes.create_string_buffer(16384)
    check(lib().mmc_config_format(ctypes.byref(cfg), buf, len(buf)))
    return buf.value.decode()


def padded_dims(cfg):
    out = (ctypes.c_int * 3)()
    check(lib().mmc_padded_dims(ctypes.byref(cfg), out))
    return tuple(out)


def transform_dims(cfg):
    """The grid the demag transforms run on (mmc_transform_dims; no device call)."""
    out = (ctypes.c_int * 3)()
    check(lib().mmc_transform_dims(ctypes.byref(cfg), out))
    return tuple(out)


def ovf_read(path, nx, ny, nz, dx, dy, dz):
    n = nx * ny * nz
    m = np.zeros((3, n))
    check(lib().mmc_ovf_read(str(path).encode(), nx, ny, nz, dx, dy, dz, dptr(m[0]), dptr(m[1]), dptr(m[2])))
    return m


def ovf_write(path, m, nx, ny, nz, dx, dy, dz, fmt=OVF_BINARY4, title="m"):
    m = np.ascontiguousarray(m, dtype=np.float64).reshape(3, -1)
    check(lib().mmc_ovf_write(str(path).encode(), nx, ny, nz, dx, dy, dz, dptr(m[0]), dptr(m[1]), dptr(m[2]),
                              fmt, title.encode()))


def philox_device(ctr, k0, k1, device=0):
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    n = ctr.shape[0]
    out = np.zeros((n, 4), np.uint32)
    outc = np.zeros((n, 4), np.uint32)
    check(lib().mmc_selftest_philox(device, n, ctr.ctypes.data_as(_u32p), k0, k1, out.ctypes.data_as(_u32p),
                                    outc.ctypes.data_as(_u32p)))
    return out, outc


class Lattice:
    """One device lattice (an mmc_handle)."""

    def __init__(self, cfg, device=0):
        self.cfg = cfg
        self.h = ctypes.c_void_p()
        check(lib().mmc_create(ctypes.byref(cfg), device, ctypes.byref(self.h)))
        self.n = cfg.nx * cfg.ny * cfg.nz
        self.pdims = padded_dims(cfg)

    def close(self):
        if self.h:
            lib().mmc_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_random(self, seed):
        check(lib().mmc_init_random(self.h, seed))

    def set_m(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(3, self.n)
        check(lib().mmc_set_m(self.h, dptr(m[0]), dptr(m[1]), dptr(m[2])))

    def get_m(self):
        m = np.zeros((3, self.n))
        check(lib().mmc_get_m(self.h, dptr(m[0]), dptr(m[1]), dptr(m[2])))
        return m

    def build_demag(self, cache_dir=""):
        check(lib().mmc_build_demag(self.h, cache_dir.encode() if cache_dir else None))

    def set_stream(self, stream):
        """Enqueue the lattice's work on a caller's cudaStream_t (an int
        handle, e.g. torch.cuda.Stream().cuda_stream); None: its own stream."""
        check(lib().mmc_set_stream(self.h, ctypes.c_void_p(stream) if stream else None))

    def tensor(self):
        np_ = self.pdims[0] * self.pdims[1] * self.pdims[2]
        k = np.zeros((6, np_))
        check(lib().mmc_get_tensor(self.h, dptr(k)))
        return k

    def self_tensor(self):
        k = np.zeros(6)
        check(lib().mmc_self_tensor(self.h, dptr(k)))
        return k

    def compute_demag(self):
        check(lib().mmc_compute_demag(self.h))

    def field(self, term):
        f = np.zeros((3, self.n))
        check(lib().mmc_get_field(self.h, term, dptr(f[0]), dptr(f[1]), dptr(f[2])))
        return f

    def energy(self):
        o = Observables()
        check(lib().mmc_energy(self.h, ctypes.byref(o)))
        return o

    def run_sweeps(self, T, stage, sweep0, nsweeps):
        check(lib().mmc_run_sweeps(self.h, float(T), stage, sweep0, nsweeps))

    def run_anneal(self, outdir, verbose=False):
        check(lib().mmc_run_anneal(self.h, str(outdir).encode(), 1 if verbose else 0))

    def engine(self):
        """(engine, band, blocks) actually used for sweeps."""
        out = (ctypes.c_int * 3)()
        check(lib().mmc_engine_info(self.h, out))
        return tuple(out)

    def last_run_ms(self):
        v = ctypes.c_double()
        check(lib().mmc_last_run_ms(self.h, ctypes.byref(v)))
        return v.value

    def profile_sweeps(self, T, stage, sweep0, nsweeps):
        out = np.zeros(3)
        check(lib().mmc_profile_sweeps(self.h, float(T), stage, sweep0, nsweeps, dptr(out)))
        return out

    def profile_fused(self, T, stage, sweep0, nsweeps):
        """Phase timestamps (ns) of the fused engine: array [16 sweeps, 9 points, 2 CTAs]."""
        out = np.zeros(16 * 9 * 2, dtype=np.uint64)
        check(lib().mmc_profile_fused(self.h, float(T), stage, sweep0, nsweeps,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        return out.reshape(16, 9, 2)

    def request_stop(self):
        lib().mmc_request_stop(self.h)

    def demag_scratch_bytes(self):
        b = ctypes.c_size_t()
        check(lib().mmc_demag_scratch_bytes(self.h, ctypes.byref(b)))
        return b.value

    def demag_apply(self, mdev, hdev, scratch, scratch_bytes, stream=None):
        check(lib().mmc_demag_apply(self.h, mdev, hdev, scratch, scratch_bytes, stream))

    def grad(self, with_m=True):
        """(dE/dm as float64 (3, n) or None, dE/d(Aex, Dind, Ku1, Ms, Bx, By, Bz))."""
        g = np.zeros((3, self.n)) if with_m else None
        dp = np.zeros(7)
        check(lib().mmc_grad(self.h, dptr(g) if with_m else None, dptr(dp)))
        return g, dp

    def relax(self, torque_tol=1e-6, max_iter=100000):
        """Projected-gradient relaxation; returns (updates, final max torque)."""
        it = ctypes.c_longlong()
        tq = ctypes.c_double()
        check(lib().mmc_relax(self.h, float(torque_tol), int(max_iter), ctypes.byref(it), ctypes.byref(tq)))
        return it.value, tq.value

    def demag_apply_static(self, mdev, hdev, stream=None):
        """mmc_demag_apply with the spectrum in the library's static device
        array (no allocation; the tensor must be built already)."""
        check(lib().mmc_demag_apply_static(self.h, mdev, hdev, stream))


def header_functions(header=HEADER):
    """Names of the functions declared in include/mmc.h."""
    import re
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mmc_[a-z0-9_]+)\s*\(", text)))


class Batch:
    """Replicas of one geometry advanced together (an mmc_batch)."""

    def __init__(self, cfgs, device=0):
        arr = (Config * len(cfgs))(*cfgs)
        self.h = ctypes.c_void_p()
        check(lib().mmc_batch_create(arr, len(cfgs), device, ctypes.byref(self.h)))
        self.R = len(cfgs)
        self.n = cfgs[0].nx * cfgs[0].ny * cfgs[0].nz

    def close(self):
        if self.h:
            lib().mmc_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_demag(self, cache_dir=""):
        check(lib().mmc_batch_build_demag(self.h, cache_dir.encode() if cache_dir else None))

    def set_stream(self, stream):
        """As Lattice.set_stream, for the batch's work."""
        check(lib().mmc_batch_set_stream(self.h, ctypes.c_void_p(stream) if stream else None))

    def set_temperatures(self, T):
        T = np.ascontiguousarray(T, dtype=np.float64)
        check(lib().mmc_batch_set_temperatures(self.h, dptr(T)))

    def temperatures(self):
        T = np.zeros(self.R)
        check(lib().mmc_batch_get_temperatures(self.h, dptr(T)))
        return T

    def set_ladders(self, replicas, temps, swap_interval, seed):
        rep = np.ascontiguousarray(replicas, dtype=np.int32)
        tp = np.ascontiguousarray(temps, dtype=np.float64)
        nl, K = rep.shape
        check(lib().mmc_batch_set_ladders(self.h, nl, K, rep.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          dptr(tp), swap_interval, seed))
        self._ladder_shape = rep.shape

    def ladder_state(self):
        rep = np.zeros(self._ladder_shape, np.int32)
        cnt = np.zeros(2, np.uint64)
        check(lib().mmc_batch_ladder_state(self.h, rep.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                           cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        return rep, cnt

    def run_sweeps(self, stage, sweep0, nsweeps):
        check(lib().mmc_batch_run_sweeps(self.h, stage, sweep0, nsweeps))

    def last_run_ms(self):
        v = ctypes.c_double()
        check(lib().mmc_batch_last_run_ms(self.h, ctypes.byref(v)))
        return v.value

    def profile_sweeps(self, stage, sweep0, nsweeps):
        out = np.zeros(5)
        check(lib().mmc_batch_profile_sweeps(self.h, stage, sweep0, nsweeps, dptr(out)))
        return out

    def autotune(self, sweeps=8):
        """Times every launch shape for `sweeps` sweeps, keeps the fastest;
        returns (best ms per sweep, candidates tried)."""
        ms = ctypes.c_double()
        n = ctypes.c_int()
        check(lib().mmc_batch_autotune(self.h, int(sweeps), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_launch_shape(self, shape):
        arr = (ctypes.c_int * 10)(*[int(v) for v in shape])
        check(lib().mmc_batch_set_launch_shape(self.h, arr))

    def launch_shape(self):
        out = (ctypes.c_int * 10)()
        check(lib().mmc_batch_launch_shape(self.h, out))
        return tuple(out)

    def energy(self):
        out = (Observables * self.R)()
        check(lib().mmc_batch_energy(self.h, out))
        return list(out)

    def set_m(self, r, m):
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(3, self.n)
        check(lib().mmc_batch_set_m(self.h, r, dptr(m[0]), dptr(m[1]), dptr(m[2])))

    def get_m(self, r):
        m = np.zeros((3, self.n))
        check(lib().mmc_batch_get_m(self.h, r, dptr(m[0]), dptr(m[1]), dptr(m[2])))
        return m


class Farm:
    """Batches of different lattice sizes advanced together (mmc_farm_*); the
    batches stay owned by the caller."""

    def __init__(self, batches):
        self.batches = list(batches)
        arr = (ctypes.c_void_p * len(self.batches))(*[b.h.value for b in self.batches])
        h = ctypes.c_void_p()
        check(lib().mmc_farm_create(arr, len(self.batches), ctypes.byref(h)))
        self.h = h

    def run_sweeps(self, stage, sweep0, nsweeps):
        check(lib().mmc_farm_run_sweeps(self.h, stage, sweep0, nsweeps))

    def last_run_ms(self):
        v = ctypes.c_double()
        check(lib().mmc_farm_last_run_ms(self.h, ctypes.byref(v)))
        return v.value

    def close(self):
        if self.h:
            lib().mmc_farm_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
