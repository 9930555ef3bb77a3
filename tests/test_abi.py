"""The C-ABI library loads and exports every symbol include/mmc.h declares;
the CLI handles its arguments.  No GPU work here."""
import ctypes
import os
import subprocess

import pytest


def test_exports_every_declared_symbol(M):
    L = M.lib()
    names = M.header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_constants(M):
    L = M.lib()
    assert L.mmc_abi_version() == 2
    assert L.mmc_config_size() == ctypes.sizeof(M.Config)
    assert L.mmc_status_string(0) == b"ok"
    assert L.mmc_status_string(7) == b"interrupted"


def test_defaults_are_the_readme_example(M):
    c = M.Config.defaults()
    assert (c.nx, c.ny, c.nz, c.pbc_x, c.pbc_y, c.pbc_z) == (256, 256, 1, 20, 20, 0)
    assert c.precision == 32 and c.cal_demag_flag == 1


def test_null_arguments_are_rejected(M):
    L = M.lib()
    assert L.mmc_create(None, 0, None) == M.ERR_INVALID
    assert b"null" in L.mmc_last_error()
    assert L.mmc_get_m(None, None, None, None) == M.ERR_INVALID
    assert L.mmc_set_stream(None, None) == M.ERR_INVALID
    assert L.mmc_batch_set_stream(None, None) == M.ERR_INVALID
    st = ctypes.c_int(-1)
    # the self-tests check their arguments before touching a device
    assert L.mmc_selftest_mbar_timeout(0, 0, ctypes.byref(st)) == M.ERR_INVALID
    assert L.mmc_selftest_mbar_timeout(0, 2_000_000_000, ctypes.byref(st)) == M.ERR_INVALID
    assert L.mmc_selftest_mbar_timeout(0, 1000, None) == M.ERR_INVALID
    assert st.value == -1


def test_create_validates_config_before_touching_a_device(M):
    c = M.Config.defaults(nx=0)
    h = ctypes.c_void_p()
    assert M.lib().mmc_create(ctypes.byref(c), 0, ctypes.byref(h)) == M.ERR_CONFIG
    # 2^31 cells or more: indices are 32-bit inside the kernels
    for dims in ((65536, 32768, 1), (2048, 2048, 512)):
        c = M.Config.defaults(nx=dims[0], ny=dims[1], nz=dims[2])
        assert M.lib().mmc_create(ctypes.byref(c), 0, ctypes.byref(h)) == M.ERR_CONFIG, dims
        assert b"2^31" in M.lib().mmc_last_error() or b"cells" in M.lib().mmc_last_error()


def test_cli_usage(M):
    cli = os.path.join(M.HERE, "bin", "mmc")
    r = subprocess.run([cli], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=60)
    assert r.returncode == 0 and "need input file" in r.stdout


def test_cli_bad_ini(M, tmp_path):
    cli = os.path.join(M.HERE, "bin", "mmc")
    p = tmp_path / "x.ini"
    p.write_text("nx = 1\n")
    r = subprocess.run([cli, str(p), "-gpu=0"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=60)
    assert r.returncode == 2 and "missing keys" in r.stderr


def test_cli_bad_farm_list(M, tmp_path):
    cli = os.path.join(M.HERE, "bin", "mmc")
    p = tmp_path / "x.ini"
    p.write_text("nx = 1\n")
    for arg in ("-farm-Bz=0.1,abc", "-farm-D=", "-farm-Bz=0.1,,0.2", "-farm-seeds=0", "-farm-seeds=",
                "-farm-seeds=3x", "-farm-seeds=70000"):
        r = subprocess.run([cli, str(p), arg], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                           timeout=60)
        assert r.returncode == 1 and "Invalid command line parameter" in r.stdout, arg
