"""Energy gradient (adjoint) and projected-gradient relaxation on the GPU.

Checked three ways: against the FP64 oracle gradient (which convolves with
K(r) and K(-r) explicitly), against central finite differences of the GPU's
own energy, and -- for the relaxation -- by the oracle's torque of the final
state.  The torch.autograd.Function lives here, in the test harness only."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CFG0 = dict(ms=1.6e6, Aex=16e-12, Dind=6e-3, Ku1=2e6, anisUx=0, anisUy=0, anisUz=1, Bextx=0, Bexty=0, Bextz=0.3,
            dx=1e-9, dy=1e-9, dz=0.8e-9)


def cfg(M, **kw):
    base = dict(CFG0, nx=16, ny=12, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=64)
    base.update(kw)
    return M.Config.defaults(**base)


def lattice_with(M, c, m):
    lat = M.Lattice(c)
    lat.set_m(m)
    return lat


GEOMS = [dict(),  # even periodic axes: the tensor is not exactly symmetric
         dict(nx=10, ny=7, nz=3, pbc_x=0, pbc_y=0, pbc_z=0, Bextx=0.05, anisUx=0.3),
         dict(nx=9, ny=8, pbc_x=1, pbc_y=0, Dind=-3e-3)]


@pytest.mark.parametrize("geom", GEOMS)
@pytest.mark.parametrize("prec", [64, 32])
def test_grad_matches_oracle(M, O, geom, prec):
    c = cfg(M, precision=prec, **geom)
    c64 = cfg(M, precision=64, **geom)
    m = O.init_random(c64, 11)
    with lattice_with(M, c, m) as lat:
        g, dp = lat.grad()
        k6 = lat.tensor()
        m_used = lat.get_m()  # rounded to the working precision
    go, dpo = O.grad(c64, k6, m_used)
    tol = 1e-12 if prec == 64 else 2e-5
    assert np.abs(g - go).max() <= tol * np.abs(go).max()
    for k in range(7):
        assert dp[k] == pytest.approx(dpo[k], rel=tol, abs=tol * np.abs(dpo).max())


def test_grad_demag_adjoint_is_symmetrised(M, O):
    """On an even periodic lattice K(r) != K(-r) by the far image; the gradient
    uses (K + K')/2, not K alone."""
    c = cfg(M, nx=6, ny=6, pbc_x=1, pbc_y=1, Aex=0, Dind=0, Ku1=0, Bextz=0)
    m = O.init_random(c, 5)
    with lattice_with(M, c, m) as lat:
        g, _ = lat.grad()
        lat.compute_demag()
        hd = lat.field(M.TERM_DEMAG)
    V = c.dx * c.dy * c.dz
    mu0 = 4e-7 * np.pi
    g_plain = -mu0 * c.ms * V * hd  # K alone
    go, _ = O.grad(c, O.tensor(c), m)
    assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()
    assert np.abs(g_plain - go).max() > 1e3 * np.abs(g - go).max()


def energy_of(lat, m):
    lat.set_m(m)
    return lat.energy().e_total


def test_grad_finite_differences_256(M, O):
    """Config-4 check: 256x256x1, config-0 material, random m from seed 11,
    central differences with step 1e-6 along 64 random unit directions."""
    c = cfg(M, nx=256, ny=256, pbc_x=20, pbc_y=20)
    m = O.init_random(c, 11)
    rng = np.random.default_rng(4)
    with lattice_with(M, c, m) as lat:
        g, _ = lat.grad()
        worst = 0.0
        for _ in range(64):
            v = rng.normal(size=m.shape)
            v /= np.linalg.norm(v)
            eps = 1e-6
            fd = (energy_of(lat, m + eps * v) - energy_of(lat, m - eps * v)) / (2 * eps)
            an = float((g * v).sum())
            worst = max(worst, abs(fd - an) / np.linalg.norm(g))
    # rounding of the energy differences, ~1e-16 |E| / eps, is ~1e-8 |g| here
    assert worst < 1e-6


def test_param_grad_finite_differences(M, O, tmp_path):
    base = dict(nx=12, ny=10, pbc_x=2, pbc_y=1, Bextx=0.02, anisUx=0.2)
    c = cfg(M, **base)
    m = O.init_random(c, 3)
    with lattice_with(M, c, m) as lat:
        lat.build_demag(str(tmp_path))
        _, dp = lat.grad()
    names = ["Aex", "Dind", "Ku1", "ms", "Bextx", "Bexty", "Bextz"]
    for k, name in enumerate(names):
        v0 = getattr(c, name)
        h = 1e-6 * max(abs(v0), 1e-2)
        e = []
        for sgn in (1, -1):
            ck = cfg(M, tensor_cache=str(tmp_path), **dict(base, **{name: v0 + sgn * h}))
            with lattice_with(M, ck, m) as lk:
                e.append(lk.energy().e_total)
        fd = (e[0] - e[1]) / (2 * h)
        assert fd == pytest.approx(dp[k], rel=1e-4), name


def test_fp32_gradient_error_against_fp64(M, O):
    c32 = cfg(M, nx=64, ny=64, precision=32)
    c64 = cfg(M, nx=64, ny=64, precision=64)
    m = O.init_random(c64, 11)
    with lattice_with(M, c32, m) as a, lattice_with(M, c64, m) as b:
        g32, p32 = a.grad()
        g64, p64 = b.grad()
    assert np.abs(g32 - g64).max() <= 1e-5 * np.abs(g64).max()
    assert np.allclose(p32, p64, rtol=1e-5, atol=1e-5 * np.abs(p64).max())


def test_autograd_function(M, O):
    torch = pytest.importorskip("torch")

    class Energy(torch.autograd.Function):
        """E(m) through the C ABI; backward through mmc_grad."""

        @staticmethod
        def forward(ctx, m, lat):
            lat.set_m(m.detach().cpu().numpy())
            ctx.lat = lat
            return torch.tensor(lat.energy().e_total, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            g, _ = ctx.lat.grad()
            return gout * torch.from_numpy(g), None

    c = cfg(M, nx=8, ny=8)
    m0 = O.init_random(c, 2)
    with M.Lattice(c) as lat:
        m = torch.tensor(m0, requires_grad=True)
        e = Energy.apply(m, lat)
        (gm,) = torch.autograd.grad(e, m)
        go, _ = O.grad(c, lat.tensor(), m0)
    assert np.abs(gm.numpy() - go).max() <= 1e-12 * np.abs(go).max()


@pytest.mark.parametrize("geom", [dict(nx=32, ny=32, pbc_x=20, pbc_y=20),
                                  dict(nx=12, ny=10, nz=2, pbc_x=0, pbc_y=0, pbc_z=0)])
def test_relaxation_reaches_torque_tolerance(M, O, geom):
    c = cfg(M, **geom)
    with M.Lattice(c) as lat:
        lat.init_random(11)
        lat.run_sweeps(300.0, 0, 0, 200)  # a thermal state to relax from
        e0 = lat.energy().e_total
        it, tq = lat.relax(1e-6, 200000)
        m = lat.get_m()
        e1 = lat.energy().e_total
        k6 = lat.tensor()
    assert tq < 1e-6 and it > 0
    assert e1 < e0
    assert np.abs(np.linalg.norm(m, axis=0) - 1).max() < 1e-12
    # the oracle's torque of the final state
    g, _ = O.grad(c, k6, m)
    V = c.dx * c.dy * c.dz
    H = -g / (4e-7 * np.pi * c.ms * V)
    torque = np.linalg.norm(np.cross(m.T, H.T), axis=1) / c.ms
    assert torque.max() < 1.01e-6
