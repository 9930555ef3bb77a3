"""Host-side logic of libmmc that needs no GPU: ini parsing, config echo,
padding rule, OVF read/write."""
import os
import struct

import numpy as np
import pytest

README_INI = """nx = 256
ny = 256
nz = 1
dx = 1e-9
dy = 1e-9
dz = 0.8e-9

Bextx = 0
Bexty = 0
Bextz = 0.3

pbc_x = 20
pbc_y = 20
pbc_z = 0

ms = 1.6e6
Aex = 16e-12
Dind = 6e-3

anisUx = 0
anisUy = 0
anisUz = 1
Ku1 = 2e6

use_random_init = true
randomseed = 256
ovf_filename = B_0_175_D_5_500_nx_100_ny_58_r_15_1.ovf

Temperature_start = 1400
Temperature_end = 40
Temperature_step = 0.90
Temperature_use_exp = true

circle_per_stage  = 100000
terminal_output_period = 10001
energy_output_period = 10001
ms_output_period = 10001

rand_block_size = 40

cal_demag_flag = true
"""


def write(tmp_path, text, name="cfg.ini"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_readme_ini(M, tmp_path):
    c = M.load_ini(write(tmp_path, README_INI))
    assert (c.nx, c.ny, c.nz) == (256, 256, 1)
    assert (c.dx, c.dy, c.dz) == (1e-9, 1e-9, 0.8e-9)
    assert (c.pbc_x, c.pbc_y, c.pbc_z) == (20, 20, 0)
    assert c.ms == 1.6e6 and c.Aex == 16e-12 and c.Dind == 6e-3 and c.Ku1 == 2e6
    assert c.use_random_init == 1 and c.randomseed == 256
    assert c.ovf_filename == b"B_0_175_D_5_500_nx_100_ny_58_r_15_1.ovf"
    assert c.Temperature_use_exp == 1 and c.Temperature_step == 0.9
    assert c.circle_per_stage == 100000 and c.energy_output_period == 10001
    assert c.rand_block_size == 40 and c.cal_demag_flag == 1
    assert c.precision == 32 and c.use_reference_pi == 0
    assert M.padded_dims(c) == (256, 256, 1)
    echo = M.format_config(c)
    assert "nx: 256" in echo and "cal_demag_flag: 1" in echo and "ovf_filename: B_0_175" in echo


def test_optional_keys(M, tmp_path):
    c = M.load_ini(write(tmp_path, README_INI + "precision = fp64\novf_format = text\nuse_reference_pi = 1\n"
                                                "tensor_cache = /tmp/cache\n"))
    assert c.precision == 64 and c.ovf_format == M.OVF_TEXT and c.use_reference_pi == 1
    assert c.tensor_cache == b"/tmp/cache"
    c = M.load_ini(write(tmp_path, README_INI + "tensor_far_radius = 32\nsweep_engine = kernels\n"))
    assert c.tensor_far_radius == 32 and c.sweep_engine == M.ENGINE_KERNELS
    assert M.load_ini(write(tmp_path, README_INI)).tensor_far_radius == 0  # reference behaviour by default


def test_comments_sections_and_bools(M, tmp_path):
    text = "; comment\n# another\n[run]\n" + README_INI.replace("use_random_init = true", "use_random_init = 0")
    c = M.load_ini(write(tmp_path, text))
    assert c.use_random_init == 0


@pytest.mark.parametrize("mutate,needle", [
    (lambda s: s.replace("nx = 256\n", ""), "missing keys: nx"),
    (lambda s: s + "nxx = 3\n", "unknown key nxx"),
    (lambda s: s.replace("nx = 256", "nx = abc"), "bad value for nx"),
    (lambda s: s + "nx = 4\n", "duplicate key nx"),
    (lambda s: s.replace("Temperature_step = 0.90", "Temperature_step = 1.5"), "Temperature_step"),
    (lambda s: s.replace("ms = 1.6e6", "ms = 0"), "ms must be"),
    (lambda s: s.replace("use_random_init = true", "use_random_init = maybe"), "bad value"),
    (lambda s: s + "precision = 16\n", "precision"),
    (lambda s: s.replace("dz = 0.8e-9", "dz = 0.8e-9 junk"), "bad value for dz"),
    (lambda s: s + "tensor_far_radius = 5\n", "tensor_far_radius"),
])
def test_ini_errors(M, tmp_path, mutate, needle):
    with pytest.raises(M.MmcError) as ei:
        M.load_ini(write(tmp_path, mutate(README_INI)))
    assert ei.value.status == M.ERR_CONFIG
    assert needle in str(ei.value)


def test_missing_ini_file(M, tmp_path):
    with pytest.raises(M.MmcError) as ei:
        M.load_ini(tmp_path / "nope.ini")
    assert ei.value.status == M.ERR_IO


def test_padding_rule(M):
    c = M.Config.defaults(nx=5, ny=4, nz=8, pbc_x=0, pbc_y=-1, pbc_z=0)
    assert M.padded_dims(c) == (9, 4, 15)


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_ovf_roundtrip(M, tmp_path, fmt):
    nx, ny, nz = 5, 3, 2
    rng = np.random.default_rng(fmt)
    m = rng.normal(size=(3, nx * ny * nz))
    m /= np.linalg.norm(m, axis=0)
    p = tmp_path / "a.ovf"
    M.ovf_write(p, m, nx, ny, nz, 1e-9, 2e-9, 3e-9, fmt=fmt)
    r = M.ovf_read(p, nx, ny, nz, 1e-9, 2e-9, 3e-9)
    if fmt == 0:
        np.testing.assert_array_equal(r, m.astype(np.float32).astype(np.float64))
    else:
        np.testing.assert_array_equal(r, m)
    head = p.read_bytes()[:200].decode(errors="replace")
    assert head.startswith("# OOMMF OVF 2.0")


def test_ovf_step_tolerance_and_mismatch(M, tmp_path):
    m = np.ones((3, 4))
    p = tmp_path / "b.ovf"
    M.ovf_write(p, m, 2, 2, 1, 1e-9, 1e-9, 1e-9, fmt=1)
    M.ovf_read(p, 2, 2, 1, 1e-9 * (1 + 1e-6), 1e-9, 1e-9)  # within 1e-5 relative
    with pytest.raises(M.MmcError) as ei:
        M.ovf_read(p, 2, 2, 1, 1.1e-9, 1e-9, 1e-9)
    assert ei.value.status == M.ERR_IO
    with pytest.raises(M.MmcError):
        M.ovf_read(p, 4, 1, 1, 1e-9, 1e-9, 1e-9)


def test_ovf1_big_endian(M, tmp_path):
    """OVF 1.0 binary data is big-endian (OOMMF / mumax3 'ovf1' output)."""
    nx, ny, nz = 2, 2, 1
    vals = np.arange(12, dtype=np.float64) / 10
    head = ("# OOMMF: rectangular mesh v1.0\n# Segment count: 1\n# Begin: Segment\n# Begin: Header\n"
            "# Title: m\n# meshtype: rectangular\n# meshunit: m\n# xstepsize: 1e-9\n# ystepsize: 1e-9\n"
            "# zstepsize: 1e-9\n# xnodes: 2\n# ynodes: 2\n# znodes: 1\n# valuemultiplier: 1\n# End: Header\n"
            "# Begin: Data Binary 8\n")
    data = struct.pack(">d", 123456789012345.0) + struct.pack(">12d", *vals)
    p = tmp_path / "c.ovf"
    p.write_bytes(head.encode() + data + b"\n# End: Data Binary 8\n# End: Segment\n")
    r = M.ovf_read(p, nx, ny, nz, 1e-9, 1e-9, 1e-9)
    np.testing.assert_array_equal(r.T.ravel(), vals)


def test_ovf_text_with_comments(M, tmp_path):
    head = ("# OOMMF OVF 2.0\n# Segment count: 1\n# Begin: Segment\n# Begin: Header\n# meshtype: rectangular\n"
            "# xnodes: 2\n# ynodes: 1\n# znodes: 1\n# xstepsize: 1e-9 # comment\n# ystepsize: 1e-9\n"
            "# zstepsize: 1e-9\n# valuedim: 3\n# End: Header\n# Begin: Data Text\n"
            "0 0 1\n# inline comment line\n1 0 0\n# End: Data Text\n# End: Segment\n")
    p = tmp_path / "d.ovf"
    p.write_text(head)
    r = M.ovf_read(p, 2, 1, 1, 1e-9, 1e-9, 1e-9)
    np.testing.assert_array_equal(r, [[0, 1], [0, 0], [1, 0]])


@pytest.mark.parametrize("bad", ["garbage\n", "# OOMMF OVF 2.0\n# xnodes: 1\n", ])
def test_ovf_malformed(M, tmp_path, bad):
    p = tmp_path / "e.ovf"
    p.write_text(bad)
    with pytest.raises(M.MmcError) as ei:
        M.ovf_read(p, 1, 1, 1, 1e-9, 1e-9, 1e-9)
    assert ei.value.status == M.ERR_IO


def test_ovf_truncated_binary(M, tmp_path):
    m = np.ones((3, 8))
    p = tmp_path / "f.ovf"
    M.ovf_write(p, m, 2, 2, 2, 1e-9, 1e-9, 1e-9, fmt=0)
    b = p.read_bytes()
    p.write_bytes(b[: len(b) // 2])
    with pytest.raises(M.MmcError):
        M.ovf_read(p, 2, 2, 2, 1e-9, 1e-9, 1e-9)


def _interop():
    import importlib.util
    p = os.path.join(os.path.dirname(__file__), "golden", "make_ovf_interop.py")
    spec = importlib.util.spec_from_file_location("make_ovf_interop", p)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name,kind", [("ovf2_b4_desc.ovf", "m32"), ("ovf2_b8_comments.ovf", "M64"),
                                       ("ovf1_b4_bigendian.omf", "m32xMS"), ("ovf2_text_spacing.ovf", "m64")])
def test_ovf_interop_files(M, name, kind):
    """OVF files laid out as other codes write them (tests/golden/make_ovf_interop.py,
    from the OVF 2.0 / 1.0 format descriptions): Desc and "##" comment lines,
    lower-case data tags, OVF 1.0 big-endian data with a value multiplier,
    irregular text spacing.  Values as stored (times the OVF 1.0 multiplier)."""
    G = _interop()
    path = os.path.join(os.path.dirname(__file__), "golden", "ovf_interop", name)
    got = M.ovf_read(path, G.NX, G.NY, G.NZ, G.DX, G.DY, G.DZ)
    f = G.field()
    want = {"m32": f.astype(np.float32).astype(np.float64), "m64": f, "M64": G.MS * f,
            "m32xMS": G.MS * f.astype(np.float32).astype(np.float64)}[kind]
    assert np.array_equal(got, want)
