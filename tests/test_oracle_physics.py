"""Physics identities of the oracle's energy, fields and Metropolis sweep."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def cfg_small(M, **kw):
    base = dict(nx=5, ny=5, nz=2, dx=1e-9, dy=1.1e-9, dz=0.8e-9, pbc_x=1, pbc_y=0, pbc_z=0, precision=64,
                randomseed=11, Bextx=0.05, Bexty=-0.02, Bextz=0.3, anisUx=0.2, anisUy=0.1, anisUz=1.0)
    base.update(kw)
    return M.Config.defaults(**base)


def test_fft_demag_equals_direct_sum(M, O):
    for kw in [dict(), dict(nx=4, ny=4, nz=1, pbc_x=2, pbc_y=2), dict(nx=3, ny=3, nz=3, pbc_x=0, pbc_y=0),
               dict(nx=5, ny=3, nz=1, pbc_x=-1, pbc_y=1)]:
        cfg = cfg_small(M, **kw)
        k = O.tensor(cfg)
        m = O.init_random(cfg, 5)
        hd = O.demag_direct(cfg, k, m)
        hf = O.demag_fft(cfg, k, m)
        np.testing.assert_allclose(hf, hd, rtol=0, atol=1e-13)


def test_uniform_m_has_no_exchange_or_dmi(M, O):
    cfg = cfg_small(M, pbc_x=1, pbc_y=1, pbc_z=1)
    n = cfg.nx * cfg.ny * cfg.nz
    m = np.zeros((3, n))
    m[2] = 1
    e = O.energy(cfg, m, None)
    assert e[0] == 0.0 and abs(e[1]) < 1e-40
    assert np.abs(O.field(cfg, 0, m)).max() == 0.0


def test_energy_is_minus_half_m_dot_h(M, O):
    """Bilinear terms: E = -mu0 Ms V / 2 sum m.H for exchange, DMI, demag."""
    cfg = cfg_small(M)
    k = O.tensor(cfg)
    m = O.init_random(cfg, 3)
    hd = O.demag_direct(cfg, k, m)
    e = O.energy(cfg, m, hd)
    mu0 = 4e-7 * np.pi
    V = cfg.dx * cfg.dy * cfg.dz
    for term, idx in [(0, 0), (1, 1), (4, 4)]:
        H = O.field(cfg, term, m, hd)
        want = -0.5 * mu0 * cfg.ms * V * np.sum(m * H)
        assert abs(e[idx] - want) <= 1e-10 * abs(want) + 1e-30, term


def _exch_self(cfg, m):
    """The -m_i part of H_ex: (2Aex/mu0 Ms) * (number of bonds of i / d^2) * (-m_i)."""
    mu0 = 4e-7 * np.pi
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    per = [cfg.pbc_x != 0, cfg.pbc_y != 0, cfg.pbc_z != 0]
    d = [cfg.dx, cfg.dy, cfg.dz]
    out = np.zeros_like(m)
    for i in range(nx * ny * nz):
        c = [i % nx, (i // nx) % ny, i // (nx * ny)]
        w = 0.0
        for a, n in enumerate((nx, ny, nz)):
            for s in (-1, 1):
                v = c[a] + s
                if v < 0 or v >= n:
                    if not per[a]:
                        continue
                    v %= n
                if v == c[a]:
                    continue
                w += 1 / d[a] ** 2
        out[:, i] = -2 * cfg.Aex / (mu0 * cfg.ms) * w * m[:, i]
    return out


@pytest.mark.parametrize("kw", [dict(), dict(nx=5, ny=3, nz=1, pbc_x=2, pbc_y=2), dict(nx=3, ny=1, nz=1, pbc_x=1),
                                dict(nx=3, ny=3, nz=3, pbc_x=1, pbc_y=1, pbc_z=1), dict(nx=4, ny=4, nz=1, pbc_x=0,
                                                                                      pbc_y=0)])
def test_local_delta_e_matches_global_energy_difference(M, O, kw):
    """The sweep's local dE (kernel formula) equals E(after) - E(before) of the
    full energy for single-spin flips, demag self-term included.

    Geometries are open or periodic with odd length: on an even periodic axis the
    reference's image sum runs over [-P, P] around the +n/2 offset, which leaves
    the off-diagonal kernel at the n/2 plane non-symmetric by the farthest image
    (test_even_periodic_kernel_asymmetry_is_the_far_image)."""
    cfg = cfg_small(M, **kw)
    k = O.tensor(cfg)
    n = cfg.nx * cfg.ny * cfg.nz
    rng = np.random.default_rng(1)
    m = O.init_random(cfg, 9)
    kB = 1.3806488e-23
    T = 1e9  # accept everything: every proposal is applied
    for trial in range(3):
        m0 = m.copy()
        hd0 = O.demag_direct(cfg, k, m0)
        E0 = O.energy(cfg, m0, hd0)[:5].sum()
        acc = O.sweeps(cfg, k, T, 7, trial, 1, m, demag_mode=0)
        assert acc == n
        # undo all but one cell so that exactly one spin changed
        i = int(rng.integers(n))
        m1 = m0.copy()
        m1[:, i] = m[:, i]
        hd1 = O.demag_direct(cfg, k, m1)
        E1 = O.energy(cfg, m1, hd1)[:5].sum()
        # local formula with the fields of the unchanged neighbours
        dE = _local_dE(cfg, k, m0, hd0, i, m1[:, i])
        assert abs((E1 - E0) - dE) <= 1e-9 * (abs(E0) + abs(E1)) / n + 1e-32, (E1 - E0, dE)
        m = m0


def _local_dE(cfg, k, m, hd, i, mp_):
    mu0 = 4e-7 * np.pi
    V = cfg.dx * cfg.dy * cfg.dz
    Hex = O_field_cache(cfg, 0, m)
    n = m.shape[1]
    H_ex_nbr = Hex[:, i] - _exch_self(cfg, m)[:, i]
    H_dm = O_field_cache(cfg, 1, m)[:, i]
    u = np.array([cfg.anisUx, cfg.anisUy, cfg.anisUz])
    u = u / np.linalg.norm(u)
    B = np.array([cfg.Bextx, cfg.Bexty, cfg.Bextz])
    K0 = np.array([[k[0, 0], k[1, 0], k[2, 0]], [k[1, 0], k[3, 0], k[4, 0]], [k[2, 0], k[4, 0], k[5, 0]]])
    m_i = m[:, i]
    dm = mp_ - m_i
    h_nbr = hd[:, i] - K0 @ m_i
    dE = -mu0 * cfg.ms * V * dm @ (H_ex_nbr + H_dm)
    dE += -cfg.Ku1 * V * ((mp_ @ u) ** 2 - (m_i @ u) ** 2)
    dE += -cfg.ms * V * dm @ B
    dE += -mu0 * cfg.ms ** 2 * V * (dm @ h_nbr + 0.5 * (mp_ @ K0 @ mp_ - m_i @ K0 @ m_i))
    return dE


def O_field_cache(cfg, term, m):
    import oracle_ctypes
    return oracle_ctypes.field(cfg, term, m)


def test_high_temperature_accepts_everything(M, O):
    cfg = cfg_small(M, cal_demag_flag=0)
    m = O.init_random(cfg, 1)
    n = m.shape[1]
    assert O.sweeps(cfg, None, 1e12, 0, 0, 3, m, demag_mode=0) == 3 * n
    np.testing.assert_allclose(np.linalg.norm(m, axis=0), 1.0, atol=1e-15)


def test_sweeps_are_deterministic_and_chunkable(M, O):
    """Philox keys on (seed, stage, sweep, cell): splitting a run changes nothing."""
    cfg = cfg_small(M)
    k = O.tensor(cfg)
    a = O.init_random(cfg, 2)
    b = a.copy()
    na = O.sweeps(cfg, k, 200.0, 1, 0, 6, a, demag_mode=1)
    nb = O.sweeps(cfg, k, 200.0, 1, 0, 2, b, demag_mode=1)
    nb += O.sweeps(cfg, k, 200.0, 1, 2, 4, b, demag_mode=1)
    assert na == nb
    assert np.array_equal(a, b)


def test_fft_and_direct_sweeps_agree(M, O):
    cfg = cfg_small(M, nx=4, ny=4, nz=1, pbc_x=2, pbc_y=2)
    k = O.tensor(cfg)
    a = O.init_random(cfg, 4)
    b = a.copy()
    O.sweeps(cfg, k, 150.0, 0, 0, 10, a, demag_mode=0)
    O.sweeps(cfg, k, 150.0, 0, 0, 10, b, demag_mode=1)
    assert np.array_equal(a, b)


def test_trajectory_fixture(M, O):
    """Regression pin: the committed oracle trajectory is reproduced."""
    z = np.load(os.path.join(GOLDEN, "trajectory_fp64.npz"))
    cfg = M.Config.defaults(nx=8, ny=8, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=64, randomseed=256,
                            cal_demag_flag=1, tensor_sum=0)
    k = O.tensor(cfg)
    assert np.array_equal(k, z["k6"])
    m = O.init_random(cfg, 256)
    assert np.array_equal(m, z["m0"])
    acc = O.sweeps(cfg, k, float(z["T"][0]), int(z["stage"][0]), 0, 20, m, demag_mode=0)
    assert acc == int(z["accepted"][0])
    assert np.array_equal(m, z["m20"])


def test_topological_charge_of_a_skyrmion(M, O):
    nx = ny = 24
    cfg = M.Config.defaults(nx=nx, ny=ny, nz=1, pbc_x=1, pbc_y=1, pbc_z=0)
    x, y = np.meshgrid(np.arange(nx) - nx / 2 + 0.5, np.arange(ny) - ny / 2 + 0.5)
    r = np.hypot(x, y)
    th = np.pi * np.exp(-(r / 4.0) ** 2)  # core down, far field up
    phi = np.arctan2(y, x)
    m = np.stack([np.sin(th) * np.cos(phi), np.sin(th) * np.sin(phi), np.cos(th)]).reshape(3, -1)
    q = O.energy(cfg, m, None)[8]
    assert abs(abs(q) - 1.0) < 1e-6


def test_even_periodic_kernel_asymmetry_is_the_far_image(M, O):
    """K_xy at the x = n/2 plane of an even periodic axis is the unpaired image
    term K_xy((P + 1/2) n, y) of the reference's [-P, P] image sum; it falls off
    like the dipole field of that image."""
    vals = []
    for P in (1, 2, 4):
        cfg = M.Config.defaults(nx=6, ny=5, nz=1, dx=1e-9, dy=1e-9, dz=1e-9, pbc_x=P, pbc_y=0, pbc_z=0)
        nxp, nyp, nzp = O.padded_dims(cfg)
        k = O.tensor(cfg).reshape(6, nzp, nyp, nxp)
        vals.append(np.abs(k[1, 0, :, nxp // 2]).max())
    assert vals[0] > vals[1] > vals[2] > 0
    # dipole scaling r^-3 with r = (P + 1/2) n
    assert 0.3 < vals[0] / vals[1] / ((2.5 / 1.5) ** 3) < 3


@pytest.mark.parametrize("n,open_len", [(6, 11), (9, 32), (16, 32), (40, 128), (129, 512), (200, 399),
                                        (300, 1024), (512, 1023)])
def test_transform_dims_rule(M, n, open_len):
    """The library's transform length of an open axis of n cells: 2n - 1 kept up
    to 16, the next power of two up to 256, beyond that 2n - 1 kept when its
    prime factors are <= 31 (399 = 3 7 19, 1023 = 3 11 31) and padded when not
    (257 and 599 are primes); periodic axes are never padded."""
    c = M.Config.defaults(nx=n, ny=8, nz=1, pbc_x=0, pbc_y=3, pbc_z=0)
    assert M.padded_dims(c) == (2 * n - 1, 8, 1)
    assert M.transform_dims(c) == (open_len, 8, 1)
    assert M.transform_dims(c.copy(pbc_x=2)) == (n, 8, 1)


def _rewrap_axis(f, t, n):
    """Tensor-grid index of each transform-grid index of an axis (-1: none):
    the rule the library applies when it pads an open axis past 2n - 1."""
    out = np.full(f, -1)
    for j in range(f):
        if f == t or j <= n - 1:
            out[j] = j
        elif j >= f - (n - 1):
            out[j] = j - f + t
    return out


@pytest.mark.parametrize("kw,f", [
    (dict(nx=6, ny=5, nz=1, pbc_x=0, pbc_y=1), (16, 5, 1)),
    (dict(nx=5, ny=4, nz=3, pbc_x=0, pbc_y=0), (16, 8, 8)),
    (dict(nx=7, ny=3, nz=1, pbc_x=0, pbc_y=-1), (16, 3, 1)),
    (dict(nx=9, ny=4, nz=1, pbc_x=0, pbc_y=1), None),  # 17 > 16: the library pads x to 32
    (dict(nx=11, ny=9, nz=1, pbc_x=0, pbc_y=0), None),  # 21 -> 32, 17 -> 32
])
def test_padded_transform_grid_is_the_same_convolution(M, O, kw, f):
    """The transform grid of an open axis may be longer than the reference's
    2n - 1: the tensor re-wrapped onto it (offsets |o| <= n - 1 kept, the rest
    0) gives, by circular convolution, the direct sum of the reference's
    tensor.  f = None takes the library's own transform grid
    (mmc_transform_dims); the other cases pad every open axis to a power of
    two to exercise the re-wrap where the library would not pad."""
    cfg = cfg_small(M, **kw)
    k = O.tensor(cfg)
    t = O.padded_dims(cfg)
    n = (cfg.nx, cfg.ny, cfg.nz)
    if f is None:
        f = M.transform_dims(cfg)
        assert f != tuple(t)
    maps = [_rewrap_axis(fi, ti, ni) for fi, ti, ni in zip(f, t, n)]
    kt = k.reshape(6, t[2], t[1], t[0])  # x fastest
    kf = np.zeros((6, f[2], f[1], f[0]))
    for jz in range(f[2]):
        for jy in range(f[1]):
            for jx in range(f[0]):
                iz, iy, ix = maps[2][jz], maps[1][jy], maps[0][jx]
                if min(ix, iy, iz) >= 0:
                    kf[:, jz, jy, jx] = kt[:, iz, iy, ix]
    m = O.init_random(cfg, 3)
    mg = np.zeros((3, f[2], f[1], f[0]))
    mg[:, :n[2], :n[1], :n[0]] = m.reshape(3, n[2], n[1], n[0])
    K = np.fft.fftn(kf, axes=(1, 2, 3))
    Mh = np.fft.fftn(mg, axes=(1, 2, 3))
    ab = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4, (2, 2): 5}
    h = np.zeros_like(mg)
    for a in range(3):
        acc = sum(K[ab[tuple(sorted((a, b)))]] * Mh[b] for b in range(3))
        h[a] = np.fft.ifftn(acc, axes=(0, 1, 2)).real
    got = h[:, :n[2], :n[1], :n[0]].reshape(3, -1)
    want = O.demag_direct(cfg, k, m)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)
