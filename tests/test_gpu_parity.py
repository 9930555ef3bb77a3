"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and the
committed golden fixtures.

Tolerances: integer / bit work (Philox, decisions, FP64 tensor) bit-exact; FP64
fields and energies 1e-12 relative; FP32 fields 1e-5 relative (of the field's
largest component)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

FP64_REL = 1e-12
FP32_REL = 1e-5


def cfg(M, **kw):
    base = dict(nx=16, ny=16, nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, pbc_x=2, pbc_y=2, pbc_z=0, precision=64,
                randomseed=256, Bextx=0.02, Bexty=-0.01, Bextz=0.3, anisUx=0.1, anisUy=0.0, anisUz=1.0)
    base.update(kw)
    return M.Config.defaults(**base)


GEOMS = {
    "film16_pbc2": dict(),
    "film12x10_open": dict(nx=12, ny=10, pbc_x=0, pbc_y=0),
    "slab6x5x4_open": dict(nx=6, ny=5, nz=4, pbc_x=0, pbc_y=0, pbc_z=0),
    "odd_periodic": dict(nx=15, ny=7, nz=1, pbc_x=1, pbc_y=-1),
    "mixed_3d": dict(nx=9, ny=6, nz=3, pbc_x=1, pbc_y=0, pbc_z=1),
    "radix_7_5": dict(nx=7, ny=10, nz=2, pbc_x=2, pbc_y=1, pbc_z=0),
    # pass kernels with the two-colour tile sweep: whole periodic tiles, and
    # partial tiles on an open axis
    "tile64_kernels": dict(nx=64, ny=64, pbc_x=1, pbc_y=1, sweep_engine=1),
    "tile96x41_kernels": dict(nx=96, ny=41, pbc_x=1, pbc_y=0, sweep_engine=1),
    "open12x10_kernels": dict(nx=12, ny=10, pbc_x=0, pbc_y=0, sweep_engine=1),
}


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_philox_matches_oracle_and_curand(M, O):
    rng = np.random.default_rng(3)
    ctr = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    ctr[1] = 0xFFFFFFFF
    ours, cur = M.philox_device(ctr, 0xA4093822, 0x299F31D0)
    assert np.array_equal(ours, cur)
    for i in range(0, 4096, 97):
        assert np.array_equal(ours[i], O.philox(ctr[i], [0xA4093822, 0x299F31D0]))


@pytest.mark.parametrize("prec", [64, 32])
def test_init_matches_oracle(M, O, prec):
    c = cfg(M, nx=33, ny=17, nz=3, precision=prec)
    with M.Lattice(c) as lat:
        m = lat.get_m()
    want = O.init_random(c, 256)
    if prec == 64:
        assert np.array_equal(m, want)
    else:
        assert np.array_equal(m, want.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("case", range(4))
def test_tensor_matches_golden(M, case):
    with open(os.path.join(GOLDEN, "newell_golden.json")) as f:
        g = json.load(f)["tensors"][case]
    c = cfg(M, nx=g["nx"], ny=g["ny"], nz=g["nz"], dx=g["dx"], dy=g["dy"], dz=g["dz"], pbc_x=g["pbc"][0],
            pbc_y=g["pbc"][1], pbc_z=g["pbc"][2])
    with M.Lattice(c) as lat:
        lat.build_demag()
        k = lat.tensor()
    np.testing.assert_allclose(k, np.array(g["K"]), rtol=0, atol=5e-13)


@pytest.mark.parametrize("tensor_sum", [0, 1])
@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_tensor_bitwise_equals_oracle(M, O, geom, tensor_sum):
    """Both forms of the image sums (0: the 64 terms in the reference's order,
    one thread per point; 1: node values shared in tiles, k_newell_nodes)
    equal the oracle's same form bit for bit."""
    c = cfg(M, tensor_sum=tensor_sum, **GEOMS[geom])
    with M.Lattice(c) as lat:
        lat.build_demag()
        k = lat.tensor()
        k0 = lat.self_tensor()
    want = O.tensor(c)
    assert np.array_equal(k, want)
    assert np.array_equal(k0, want[:, 0])


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_demag_field_matches_direct_sum(M, O, geom, prec):
    c = cfg(M, precision=prec, **GEOMS[geom])
    with M.Lattice(c) as lat:
        lat.build_demag()
        m = lat.get_m()
        lat.compute_demag()
        H = lat.field(M.TERM_DEMAG)
        k = lat.tensor()
    want = c.ms * O.demag_direct(c, k, m)
    assert rel(H, want) <= (FP64_REL if prec == 64 else FP32_REL)


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("term", [0, 1, 2, 3, 5])
@pytest.mark.parametrize("geom", ["film16_pbc2", "slab6x5x4_open", "odd_periodic"])
def test_field_terms(M, O, geom, term, prec):
    c = cfg(M, precision=prec, Dind=6e-3, **GEOMS[geom])
    with M.Lattice(c) as lat:
        lat.compute_demag()
        m = lat.get_m()
        H = lat.field(term)
        k = lat.tensor()
    hd = O.demag_direct(c, k, m)
    want = O.field(c, term, m, hd)
    assert rel(H, want) <= (FP64_REL if prec == 64 else FP32_REL)


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_energy_and_observables(M, O, geom, prec):
    c = cfg(M, precision=prec, **GEOMS[geom])
    with M.Lattice(c) as lat:
        o = lat.energy()
        m = lat.get_m()
        k = lat.tensor()
    want = O.energy(c, m, O.demag_direct(c, k, m))
    got = np.array([o.e_exchange, o.e_dmi, o.e_anisotropy, o.e_zeeman, o.e_demag, *o.m, o.q])
    tol = 1e-11 if prec == 64 else 2e-5
    scale = np.abs(want[:5]).sum()
    assert np.abs(got[:5] - want[:5]).max() <= tol * scale
    assert np.abs(got[5:8] - want[5:8]).max() <= 1e-12
    assert abs(got[8] - want[8]) <= 1e-9
    assert abs(o.e_total - want[:5].sum()) <= tol * scale


@pytest.mark.parametrize("demag", [0, 1])
@pytest.mark.parametrize("geom", ["film16_pbc2", "odd_periodic", "mixed_3d", "tile64_kernels", "tile96x41_kernels",
                                  "open12x10_kernels"])
def test_fp64_decisions_bitwise_100_sweeps(M, O, geom, demag):
    """FP64 accept/reject decisions identical to the oracle's for 100 sweeps:
    the final state (every spin is its initial vector or a Philox proposal) and
    the accept count must match exactly."""
    c = cfg(M, cal_demag_flag=demag, **GEOMS[geom])
    with M.Lattice(c) as lat:
        m0 = lat.get_m()
        k = lat.tensor() if demag else None
        T = 120.0
        lat.run_sweeps(T, 4, 0, 100)
        m_gpu = lat.get_m()
        o = lat.energy()
    m = m0.copy()
    acc = O.sweeps(c, k, T, 4, 0, 100, m, demag_mode=1)
    assert o.proposed == 100 * m.shape[1]
    assert o.accepted == acc
    assert np.array_equal(m_gpu, m)


def test_trajectory_fixture(M):
    z = np.load(os.path.join(GOLDEN, "trajectory_fp64.npz"))
    c = M.Config.defaults(nx=8, ny=8, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=64, randomseed=256,
                          cal_demag_flag=1, tensor_sum=0)
    with M.Lattice(c) as lat:
        lat.build_demag()
        assert np.array_equal(lat.tensor(), z["k6"])
        assert np.array_equal(lat.get_m(), z["m0"])
        lat.run_sweeps(float(z["T"][0]), int(z["stage"][0]), 0, 20)
        assert np.array_equal(lat.get_m(), z["m20"])
        o = lat.energy()
    assert o.accepted == int(z["accepted"][0])
    e = z["e20"]
    assert abs(o.e_total - e[:5].sum()) <= 1e-11 * np.abs(e[:5]).sum()


def test_fp32_tracks_fp64_for_a_few_sweeps(M):
    """FP32 and FP64 runs share the random stream; with the same start they make
    the same decisions until a near-tie, so early states agree closely."""
    c64 = cfg(M, precision=64)
    c32 = cfg(M, precision=32)
    with M.Lattice(c64) as a, M.Lattice(c32) as b:
        b.set_m(a.get_m())
        a.run_sweeps(300.0, 0, 0, 3)
        b.run_sweeps(300.0, 0, 0, 3)
        ma, mb = a.get_m(), b.get_m()
    same = np.all(np.abs(ma - mb) < 1e-6, axis=0).mean()
    assert same > 0.99


def test_chunked_runs_equal_single_run(M):
    c = cfg(M, nx=32, ny=32, precision=32)
    with M.Lattice(c) as a, M.Lattice(c) as b:
        a.run_sweeps(250.0, 2, 0, 150)  # graph replays + tail
        for s0, ns in [(0, 10), (10, 64), (74, 76)]:
            b.run_sweeps(250.0, 2, s0, ns)
        assert np.array_equal(a.get_m(), b.get_m())


def test_demag_apply_on_device_pointers(M):
    torch = pytest.importorskip("torch")
    c = cfg(M, nx=20, ny=12, nz=2, pbc_x=1, pbc_y=0, pbc_z=0, precision=32)
    with M.Lattice(c) as lat:
        lat.compute_demag()
        want = lat.field(M.TERM_DEMAG) / c.ms
        m = lat.get_m()
        dev = torch.device("cuda:0")
        mt = torch.tensor(m, dtype=torch.float32, device=dev).contiguous()
        ht = torch.zeros_like(mt)
        nb = lat.demag_scratch_bytes()
        scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        lat.demag_apply(mt.data_ptr(), ht.data_ptr(), scratch.data_ptr(), nb, None)
        lat.compute_demag()  # same stream: orders after demag_apply
        torch.cuda.synchronize()
        got = ht.cpu().numpy().astype(np.float64)
        with pytest.raises(M.MmcError):
            lat.demag_apply(mt.data_ptr(), ht.data_ptr(), scratch.data_ptr(), nb - 1, None)
    assert rel(got, want) <= 1e-6


def test_tensor_cache_roundtrip(M, tmp_path):
    c = cfg(M, nx=10, ny=6, nz=1, pbc_x=3, pbc_y=0)
    with M.Lattice(c) as lat:
        lat.build_demag(str(tmp_path))
        k1 = lat.tensor()
    name = "cache_10_11_1-1e-09_1e-09_8e-10-3_0_0.ovf"
    f = tmp_path / name
    assert f.exists() and f.stat().st_size == 6 * 10 * 11 * 1 * 8
    raw = np.fromfile(f, dtype=np.float64).reshape(6, 10, 11, 1)  # reference layout: x slowest, z fastest
    assert np.array_equal(raw.transpose(0, 3, 2, 1).reshape(6, -1), k1)
    # a cached file is used as is: perturb it and read it back
    raw2 = raw.copy()
    raw2[5, 0, 0, 0] = 0.5
    raw2.tofile(f)
    with M.Lattice(c) as lat:
        lat.build_demag(str(tmp_path))
        k2 = lat.tensor()
    assert k2[5, 0] == 0.5 and np.array_equal(k2[:5], k1[:5])


def test_anneal_outputs(M, tmp_path):
    """The stage loop writes energy.txt ("%f %ld %g") and OVF snapshots named
    %06ld_%.2fK_%ld.ovf, clearing old images from the output folder."""
    c = cfg(M, nx=8, ny=8, precision=32, Temperature_start=100.0, Temperature_end=70.0, Temperature_step=0.9,
            circle_per_stage=20, energy_output_period=10, ms_output_period=15, terminal_output_period=7)
    out = tmp_path / "run.output"
    out.mkdir()
    (out / "old.png").write_text("x")
    (out / "keep.txt").write_text("x")
    with M.Lattice(c) as lat:
        lat.run_anneal(out)
    assert not (out / "old.png").exists() and (out / "keep.txt").exists()
    lines = (out / "energy.txt").read_text().splitlines()
    # float32 temperatures 100, 90, 81, 72.9 (> 70), four stages; energy at sweeps 0 and 10
    temps = [float(l.split()[0]) for l in lines]
    assert [l.split()[1] for l in lines] == ["0", "10"] * 4
    assert temps[::2] == pytest.approx([100.0, 90.0, 81.0, 72.9], rel=1e-6)
    snaps = sorted(p.name for p in out.glob("*.ovf"))
    assert snaps[0] == "000000_100.00K_0.ovf" and len(snaps) == 8
    assert "000001_100.00K_15.ovf" in snaps
    m = M.ovf_read(out / snaps[-1], 8, 8, 1, c.dx, c.dy, c.dz)
    np.testing.assert_allclose(np.linalg.norm(m, axis=0), 1, atol=1e-6)


def test_debug_field_dumps(M, O, tmp_path):
    """debug_h_field = 1: at every energy output the stage loop writes
    B_demag / B_anis / B_exch / B_dmi / B_effective (mu0 H, T) and E_density
    (J/m^3), as the reference's DEBUG_H_FIELD build (src/main.cu:965-1086).
    Three stages of 20 sweeps with one energy output each: the files left are
    those of the last stage's start, i.e. of the state after 40 sweeps.  They
    equal the library's own fields of that state bit for bit (FP64, Binary 8),
    and the oracle's within 1e-12; E_density sums to the total energy."""
    kw = dict(nx=12, ny=10, precision=64, Dind=6e-3, debug_h_field=1, ovf_format=M.OVF_BINARY8,
              Temperature_start=200.0, Temperature_end=150.0, Temperature_step=0.9, circle_per_stage=20,
              energy_output_period=20, ms_output_period=1000, terminal_output_period=1000)
    c = cfg(M, **kw)
    out = tmp_path / "run.output"
    out.mkdir()
    with M.Lattice(c) as lat:
        lat.build_demag()
        m0 = lat.get_m()
        k = lat.tensor()
        lat.run_anneal(out)
    mu0 = 4e-7 * np.pi
    files = {t: M.ovf_read(out / (t + ".ovf"), c.nx, c.ny, 1, c.dx, c.dy, c.dz)
             for t in ("B_demag", "B_anis", "B_exch", "B_dmi", "B_effective", "E_density")}
    terms = {"B_exch": M.TERM_EXCHANGE, "B_dmi": M.TERM_DMI, "B_anis": M.TERM_ANISOTROPY,
             "B_demag": M.TERM_DEMAG, "B_effective": M.TERM_TOTAL}
    with M.Lattice(c.copy(debug_h_field=0)) as lat:
        lat.set_m(m0)
        lat.run_sweeps(200.0, 0, 0, 20)
        lat.run_sweeps(180.0, 1, 0, 20)
        lat.compute_demag()
        m40 = lat.get_m()
        for name, term in terms.items():
            assert np.array_equal(files[name], mu0 * lat.field(term)), name
        e_total = lat.energy().e_total
    m = m0.copy()
    O.sweeps(c, k, 200.0, 0, 0, 20, m, demag_mode=1)
    O.sweeps(c, k, 180.0, 1, 0, 20, m, demag_mode=1)
    assert np.array_equal(m, m40)
    hd = O.demag_fft(c, k, m)
    for name, term in terms.items():
        want = mu0 * O.field(c, term, m, hd)
        assert rel(files[name], want) <= FP64_REL, name
    e = files["E_density"]
    assert np.array_equal(e[0], e[1]) and np.array_equal(e[0], e[2])
    V = c.dx * c.dy * c.dz
    assert abs(e[0].sum() * V - e_total) <= 1e-11 * abs(O.energy(c, m, hd)[:5]).sum()


@pytest.mark.parametrize("name", ["ovf2_b8_comments.ovf", "ovf1_b4_bigendian.omf", "ovf2_text_spacing.ovf"])
def test_initial_state_from_interop_ovf(M, name):
    """ovf_filename with use_random_init = 0: a file of M in A/m (or of m times
    an OVF 1.0 multiplier) starts the lattice at the unit vectors M / |M|; a
    file of unit vectors is taken as it is."""
    import importlib.util
    p = os.path.join(GOLDEN, "make_ovf_interop.py")
    spec = importlib.util.spec_from_file_location("make_ovf_interop", p)
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    path = os.path.join(GOLDEN, "ovf_interop", name)
    c = M.Config.defaults(nx=G.NX, ny=G.NY, nz=G.NZ, dx=G.DX, dy=G.DY, dz=G.DZ, pbc_x=1, pbc_y=1, pbc_z=0,
                          precision=64, use_random_init=0, ovf_filename=path)
    with M.Lattice(c) as lat:
        m = lat.get_m()
    raw = M.ovf_read(path, G.NX, G.NY, G.NZ, G.DX, G.DY, G.DZ)
    if name == "ovf2_text_spacing.ovf":
        assert np.array_equal(m, raw)
    else:
        np.testing.assert_allclose(m, raw / np.linalg.norm(raw, axis=0), rtol=0, atol=4e-16)


def test_stop_request_interrupts(M):
    import threading
    import time
    c = cfg(M, nx=64, ny=64, precision=32)
    with M.Lattice(c) as lat:
        lat.build_demag()
        t = threading.Timer(0.5, lat.request_stop)
        t.start()
        t0 = time.time()
        with pytest.raises(M.MmcError) as ei:
            lat.run_sweeps(300.0, 0, 0, 10 ** 7)
        t.cancel()
        assert ei.value.status == M.ERR_INTERRUPTED
        assert time.time() - t0 < 30
        lat.run_sweeps(300.0, 0, 0, 5)  # handle stays usable


def test_cli_end_to_end(M, tmp_path):
    import subprocess
    ini = tmp_path / "tiny.ini"
    text = open(os.path.join(os.path.dirname(__file__), "test_host_io.py")).read()
    body = text.split('README_INI = """')[1].split('"""')[0]
    body = (body.replace("nx = 256", "nx = 16").replace("ny = 256", "ny = 16")
            .replace("circle_per_stage  = 100000", "circle_per_stage = 50")
            .replace("Temperature_end = 40", "Temperature_end = 1100")
            .replace("pbc_x = 20", "pbc_x = 2").replace("pbc_y = 20", "pbc_y = 2"))
    ini.write_text(body)
    cli = os.path.join(M.HERE, "bin", "mmc")
    cache = tmp_path / "cache"
    cache.mkdir()
    r = subprocess.run([cli, str(ini), "-gpu=0", f'-tensorcache="{cache}"'], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "tiny.output"
    lines = (out / "energy.txt").read_text().splitlines()
    assert len(lines) == 3  # 1400, 1260, 1134 (> 1100)
    assert len(list(cache.glob("cache_16_16_1-*.ovf"))) == 1
    assert len(list(out.glob("*.ovf"))) == 3


@pytest.mark.parametrize("args,count", [(("-farm-Bz=0.1,0.4", "-farm-D=3e-3,5e-3"), 4),
                                        (("-farm-Bz=0.2", "-farm-seeds=3"), 3)])
def test_cli_parameter_farm_equals_single_runs(M, tmp_path, args, count):
    """-farm-Bz= / -farm-D= / -farm-seeds= anneal every (B_z, D) pair, as many
    seeds of each as asked, as replicas of one batch; each replica's
    energy.txt and snapshots equal those of a single CLI run of the ini with
    that B_z, D and seed."""
    import shutil
    import subprocess
    text = open(os.path.join(os.path.dirname(__file__), "test_host_io.py")).read()
    body = text.split('README_INI = """')[1].split('"""')[0]
    body = (body.replace("nx = 256", "nx = 16").replace("ny = 256", "ny = 16")
            .replace("circle_per_stage  = 100000", "circle_per_stage = 40")
            .replace("Temperature_end = 40", "Temperature_end = 1100")
            .replace("pbc_x = 20", "pbc_x = 2").replace("pbc_y = 20", "pbc_y = 2"))
    cli = os.path.join(M.HERE, "bin", "mmc")
    farm_dir = tmp_path / "farm"
    farm_dir.mkdir()
    (farm_dir / "f.ini").write_text(body)
    r = subprocess.run([cli, str(farm_dir / "f.ini"), *args],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = farm_dir / "f.output"
    rows = [l.split() for l in (out / "farm.txt").read_text().splitlines()]
    assert len(rows) == count
    base_seed = int(M.load_ini(str(farm_dir / "f.ini")).randomseed)
    for k, bz, dm, seed in rows:
        assert int(seed) == base_seed + int(k)
        single = tmp_path / f"single{k}"
        single.mkdir()
        one = (body.replace("Bextz = 0.3", f"Bextz = {bz}").replace("Dind = 6e-3", f"Dind = {dm}")
               .replace(f"randomseed = {base_seed}", f"randomseed = {seed}"))
        (single / "s.ini").write_text(one)
        r1 = subprocess.run([cli, str(single / "s.ini")], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            text=True, timeout=300)
        assert r1.returncode == 0, r1.stdout + r1.stderr
        rep = out / f"replica_{int(k):03d}"
        assert (rep / "energy.txt").read_text() == (single / "s.output" / "energy.txt").read_text()
        snaps = sorted(p.name for p in rep.glob("*.ovf"))
        assert snaps and snaps == sorted(p.name for p in (single / "s.output").glob("*.ovf"))
        for name in snaps:
            assert (rep / name).read_bytes() == (single / "s.output" / name).read_bytes()
        shutil.rmtree(single)


FILMS = {
    "periodic32": dict(nx=32, ny=32, pbc_x=2, pbc_y=2),
    "open20x12": dict(nx=20, ny=12, pbc_x=0, pbc_y=0),
    "mixed24x10": dict(nx=24, ny=10, pbc_x=1, pbc_y=0),
    "ny2_periodic": dict(nx=16, ny=2, pbc_x=1, pbc_y=1),
    "ny3_open": dict(nx=20, ny=3, pbc_x=1, pbc_y=0),
    "ny1": dict(nx=12, ny=1, pbc_x=1, pbc_y=0),
    "rect_x96": dict(nx=96, ny=6, pbc_x=1, pbc_y=-1),
    "tile64": dict(nx=64, ny=64, pbc_x=2, pbc_y=2),
    "tile96x41": dict(nx=96, ny=41, pbc_x=1, pbc_y=0),
    # open x of 200 cells: transform length 399 = 3 7 19 (kept, not padded to
    # 512, so the film engine takes it)
    "open200x24": dict(nx=200, ny=24, pbc_x=0, pbc_y=1),
}


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("film", sorted(FILMS))
def test_fused_engine_bitwise_equals_kernels(M, film, prec):
    c = cfg(M, precision=prec, **FILMS[film])
    ck = c.copy(sweep_engine=M.ENGINE_KERNELS)
    cf = c.copy(sweep_engine=M.ENGINE_FUSED)
    with M.Lattice(ck) as a, M.Lattice(cf) as b:
        assert a.engine()[0] == M.ENGINE_KERNELS and b.engine()[0] == M.ENGINE_FUSED
        a.run_sweeps(180.0, 5, 0, 37)
        b.run_sweeps(180.0, 5, 0, 37)
        oa, ob = a.energy(), b.energy()
        assert np.array_equal(a.get_m(), b.get_m())
        assert oa.accepted == ob.accepted and oa.proposed == ob.proposed
        # the demag field left behind is the one of the last sweep's start in both
        assert np.array_equal(a.field(M.TERM_DEMAG), b.field(M.TERM_DEMAG))


@pytest.mark.parametrize("band", [1, 2, 3, 5, 16])
def test_fused_band_sizes(M, band):
    c = cfg(M, nx=40, ny=30, pbc_x=1, pbc_y=1, precision=32)
    with M.Lattice(c.copy(sweep_engine=M.ENGINE_KERNELS)) as a, \
            M.Lattice(c.copy(sweep_engine=M.ENGINE_FUSED, fused_band=band)) as b:
        assert b.engine()[1] == band and b.engine()[2] == (30 + band - 1) // band
        a.run_sweeps(250.0, 1, 3, 20)
        b.run_sweeps(250.0, 1, 3, 20)
        assert np.array_equal(a.get_m(), b.get_m())


def test_fused_fp64_decisions_match_oracle(M, O):
    c = cfg(M, nx=24, ny=20, pbc_x=2, pbc_y=0, precision=64, sweep_engine=M.ENGINE_FUSED)
    with M.Lattice(c) as lat:
        m0 = lat.get_m()
        k = lat.tensor()
        lat.run_sweeps(90.0, 2, 0, 100)
        m_gpu = lat.get_m()
        o = lat.energy()
    m = m0.copy()
    acc = O.sweeps(c, k, 90.0, 2, 0, 100, m, demag_mode=1)
    assert o.accepted == acc
    assert np.array_equal(m_gpu, m)


def test_fused_long_run_spans_several_launches(M):
    c = cfg(M, nx=64, ny=64, pbc_x=1, pbc_y=1, precision=32)
    with M.Lattice(c.copy(sweep_engine=M.ENGINE_KERNELS)) as a, M.Lattice(c.copy(sweep_engine=M.ENGINE_FUSED)) as b:
        a.run_sweeps(400.0, 0, 0, 2500)
        b.run_sweeps(400.0, 0, 0, 2500)
        assert np.array_equal(a.get_m(), b.get_m())


def test_engine_auto_selection(M):
    with M.Lattice(cfg(M, nx=16, ny=16)) as lat:
        assert lat.engine()[0] == M.ENGINE_FUSED
    with M.Lattice(cfg(M, nx=6, ny=5, nz=4, pbc_x=0, pbc_y=0, pbc_z=0)) as lat:
        assert lat.engine()[0] == M.ENGINE_KERNELS
    with M.Lattice(cfg(M, nx=15, ny=8, pbc_x=1)) as lat:  # odd periodic: three colours
        assert lat.engine()[0] == M.ENGINE_KERNELS
    with pytest.raises(M.MmcError) as ei:
        M.Lattice(cfg(M, nx=15, ny=8, pbc_x=1, sweep_engine=M.ENGINE_FUSED))
    assert ei.value.status == M.ERR_UNSUPPORTED


def test_device_wait_timeout_is_reported_and_device_stays_usable(M):
    """Failure detection without a fault: a barrier wait that nothing can
    complete runs out of its poll budget, the kernel returns, the host reads
    MMC_ERR_TIMEOUT, and the next computation on the device is still right."""
    import ctypes
    st = ctypes.c_int(-1)
    M.check(M.lib().mmc_selftest_barrier_timeout(0, 4096, ctypes.byref(st)))
    assert st.value == 8  # MMC_ERR_TIMEOUT
    c = cfg(M, nx=16, ny=16, precision=64)
    with M.Lattice(c) as a:
        a.run_sweeps(200.0, 0, 0, 5)
        assert a.energy().accepted > 0


def test_mbarrier_wait_timeout_is_reported_and_device_stays_usable(M):
    """The pipelined Metropolis form's bounded wait on a transaction barrier
    that nothing completes (no copy in flight) gives up after its time limit
    (1 ms here), the host reads MMC_ERR_TIMEOUT, and the pipelined form then
    runs and reports no error."""
    import ctypes
    st = ctypes.c_int(-1)
    M.check(M.lib().mmc_selftest_mbar_timeout(0, 1000000, ctypes.byref(st)))
    assert st.value == 8  # MMC_ERR_TIMEOUT
    cfgs = [cfg(M, nx=64, ny=32, precision=32, randomseed=5 + r) for r in range(2)]
    with M.Batch(cfgs) as b:
        s = list(b.launch_shape())
        s[6] = 5
        b.set_launch_shape(s)
        b.run_sweeps(0, 0, 40)
        assert all(o.accepted > 0 for o in b.energy())


@pytest.mark.parametrize("geom", [dict(nx=16, ny=12, pbc_x=2, pbc_y=1), dict(nx=10, ny=8, nz=3, pbc_x=3, pbc_y=0,
                                                                           pbc_z=0)])
def test_far_radius_tensor_bitwise_equals_oracle(M, O, geom, tmp_path):
    """The far-field tensor terms (tensor_far_radius) are computed by the same
    expression on the GPU and in the oracle; the cache keeps them apart from
    the exact tensor's file."""
    c = cfg(M, tensor_far_radius=12, **geom)
    with M.Lattice(c) as lat:
        lat.build_demag(str(tmp_path))
        k = lat.tensor()
    assert np.array_equal(k, O.tensor(c))
    names = sorted(p.name for p in tmp_path.iterdir())
    assert len(names) == 1 and names[0].endswith("_far12.ovf")


WIDE = {
    "x512": dict(nx=512, ny=4, pbc_x=1, pbc_y=1),
    "y512_open_x": dict(nx=6, ny=512, pbc_x=0, pbc_y=1),
    "x1024": dict(nx=1024, ny=2, pbc_x=1, pbc_y=1),
    "z512": dict(nx=2, ny=3, nz=512, pbc_x=1, pbc_y=1, pbc_z=1),
}


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("geom", sorted(WIDE))
def test_wide_transforms_match_oracle(M, O, geom, prec):
    """Padded sides of 512 and 1024 (32 values per lane in the warp-level
    transforms, x passes, column passes along y and along z): demag field
    against the oracle's direct sum, and FP64 decisions bit for bit."""
    c = cfg(M, precision=prec, **WIDE[geom])
    with M.Lattice(c) as lat:
        lat.build_demag()
        m0 = lat.get_m()
        lat.compute_demag()
        H = lat.field(M.TERM_DEMAG)
        k = lat.tensor()
        lat.run_sweeps(150.0, 2, 0, 20)
        m_gpu = lat.get_m()
        acc_gpu = lat.energy().accepted
    assert rel(H, c.ms * O.demag_direct(c, k, m0)) <= (FP64_REL if prec == 64 else FP32_REL)
    if prec == 64:
        m = m0.copy()
        acc = O.sweeps(c, k, 150.0, 2, 0, 20, m, demag_mode=1)
        assert acc_gpu == acc
        assert np.array_equal(m_gpu, m)


@pytest.mark.parametrize("prec", [64, 32])
def test_open_axis_with_large_prime_padding(M, O, prec):
    """An open x axis of 40 cells: the reference's padded length 79 is a prime
    above the mixed-radix transforms' largest radix, so the transform grid is
    padded on to 128 and the tensor re-wrapped onto it.  Field against the
    oracle's direct sum on the 79-cell tensor grid; FP64 decisions bit for bit."""
    c = cfg(M, nx=40, ny=8, nz=1, pbc_x=0, pbc_y=1, precision=prec)
    assert M.padded_dims(c) == (79, 8, 1)
    with M.Lattice(c) as lat:
        lat.build_demag()
        m0 = lat.get_m()
        lat.compute_demag()
        H = lat.field(M.TERM_DEMAG)
        k = lat.tensor()
        lat.run_sweeps(150.0, 1, 0, 30)
        m_gpu = lat.get_m()
        acc_gpu = lat.energy().accepted
    assert rel(H, c.ms * O.demag_direct(c, k, m0)) <= (FP64_REL if prec == 64 else FP32_REL)
    if prec == 64:
        m = m0.copy()
        acc = O.sweeps(c, k, 150.0, 1, 0, 30, m, demag_mode=1)
        assert acc_gpu == acc
        assert np.array_equal(m_gpu, m)


def test_caller_stream(M):
    """A lattice's and a batch's work enqueued on a caller's stream (a torch
    stream here) gives the results of their own streams, in order with the
    work enqueued before the switch and after switching back; the default
    streams are refused."""
    torch = pytest.importorskip("torch")
    import ctypes
    s = torch.cuda.Stream()
    c = cfg(M, nx=32, ny=32, precision=32)
    with M.Lattice(c) as a, M.Lattice(c) as b:
        a.run_sweeps(300.0, 0, 0, 10)
        b.run_sweeps(300.0, 0, 0, 10)
        b.set_stream(s.cuda_stream)
        a.run_sweeps(300.0, 0, 10, 40)
        b.run_sweeps(300.0, 0, 10, 40)
        b.set_stream(None)
        a.run_sweeps(300.0, 0, 50, 5)
        b.run_sweeps(300.0, 0, 50, 5)
        assert np.array_equal(a.get_m(), b.get_m())
        assert a.energy().accepted == b.energy().accepted
        for bad in (1, 2):  # cudaStreamLegacy, cudaStreamPerThread
            with pytest.raises(M.MmcError):
                M.check(M.lib().mmc_set_stream(b.h, ctypes.c_void_p(bad)))
    cfgs = [cfg(M, nx=64, ny=32, precision=32, randomseed=40 + r) for r in range(3)]
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sh = list(b.launch_shape())
        sh[9] = 2  # replica parts on two streams, forked from the caller's
        a.set_launch_shape(sh)
        b.set_launch_shape(sh)
        b.set_stream(s.cuda_stream)
        a.run_sweeps(0, 0, 70)
        b.run_sweeps(0, 0, 70)
        for r in range(3):
            assert np.array_equal(a.get_m(r), b.get_m(r))
        b.set_stream(None)


DEGENERATE = {
    "cell_open": dict(nx=1, ny=1, nz=1, pbc_x=0, pbc_y=0, pbc_z=0),
    "cell_images": dict(nx=1, ny=1, nz=1, pbc_x=2, pbc_y=2, pbc_z=0),
    "x1_column": dict(nx=1, ny=7, nz=1, pbc_x=1, pbc_y=0),
    "y1_slab": dict(nx=5, ny=1, nz=3, pbc_x=0, pbc_y=0, pbc_z=0),
    "z_column": dict(nx=1, ny=1, nz=6, pbc_x=0, pbc_y=0, pbc_z=1),
}


@pytest.mark.parametrize("geom", sorted(DEGENERATE))
def test_degenerate_lattices_match_oracle(M, O, geom):
    """Lattices with axes of length 1 (a single cell, with and without
    periodic images; a one-cell-wide column along x; a 3-D slab one cell deep
    in y; a periodic column along z): the tensor bit for bit, 30 FP64 sweeps
    decision for decision and the energy against the oracle; the same
    lattices run in FP32 and stay on the unit sphere."""
    c = cfg(M, **DEGENERATE[geom])
    with M.Lattice(c) as lat:
        lat.build_demag()
        k = lat.tensor()
        m0 = lat.get_m()
        lat.run_sweeps(150.0, 2, 0, 30)
        m_gpu = lat.get_m()
        o = lat.energy()
        m_now = lat.get_m()
    assert np.array_equal(k, O.tensor(c))
    m = m0.copy()
    acc = O.sweeps(c, k, 150.0, 2, 0, 30, m, demag_mode=1)
    assert o.accepted == acc and o.proposed == 30 * m.shape[1]
    assert np.array_equal(m_gpu, m)
    want = O.energy(c, m_now, O.demag_direct(c, k, m_now))
    scale = np.abs(want[:5]).sum()
    assert abs(o.e_total - want[:5].sum()) <= 1e-11 * scale
    c32 = cfg(M, precision=32, **DEGENERATE[geom])
    with M.Lattice(c32) as lat:
        lat.run_sweeps(150.0, 2, 0, 30)
        m32 = lat.get_m()
        assert lat.energy().proposed == 30 * m32.shape[1]
    assert np.abs(np.linalg.norm(m32, axis=0) - 1.0).max() < 1e-6
