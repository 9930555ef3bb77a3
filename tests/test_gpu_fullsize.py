"""Parity at a benchmark configuration's full size: the 3-D slab of
512 x 512 x 8 cells (2 x 2 x 1 nm, 10 periodic images in x and y, open z,
Ms 1.1e6 A/m, the tensor exact within 32 cells and by the far-field expansion
beyond -- as the bench runs it).  At this size the oracle's direct sums would
take hours, so the checks are properties that hold at any size:

- the demag operator is linear (FP64, 1e-12 relative);
- it commutes with a translation along the periodic axes (FP64, 1e-12);
- the FP32 field equals the FP64 field of the same state to 1e-5 relative
  (of the field's largest component);
- the FP32 energy of a state reached by FP32 sweeps equals the FP64
  evaluation of that state to 1e-4 relative (the energy bar of the FP32
  path), and each term to 1e-4 of the total's scale.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SLAB = dict(nx=512, ny=512, nz=8, dx=2e-9, dy=2e-9, dz=1e-9, ms=1.1e6, Aex=15e-12, Dind=3e-3, Ku1=0.8e6,
            anisUx=0.0, anisUy=0.0, anisUz=1.0, Bextx=0.0, Bexty=0.0, Bextz=0.2, pbc_x=10, pbc_y=10, pbc_z=0,
            cal_demag_flag=1, randomseed=7, use_random_init=1, tensor_far_radius=32, sweep_engine=1)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def cache(tmp_path_factory):
    return str(tmp_path_factory.mktemp("slab_tensor"))


def demag(lat, M, m):
    lat.set_m(m)
    lat.compute_demag()
    return lat.field(M.TERM_DEMAG)


def test_slab_demag_linear_translation_equivariant_and_fp32(M, cache):
    c64 = M.Config.defaults(precision=64, **SLAB)
    c32 = M.Config.defaults(precision=32, **SLAB)
    shape = (3, SLAB["nz"], SLAB["ny"], SLAB["nx"])
    with M.Lattice(c64) as lat:
        lat.build_demag(cache)
        # the random start, rounded to FP32 so both precisions see one state
        m1 = lat.get_m().astype(np.float32).astype(np.float64)
        rng = np.random.default_rng(3)
        m2 = rng.normal(size=m1.shape)
        m2 /= np.linalg.norm(m2, axis=0)
        h1 = demag(lat, M, m1)
        h2 = demag(lat, M, m2)
        h12 = demag(lat, M, m1 + 2.0 * m2)
        assert rel(h12, h1 + 2.0 * h2) <= 1e-12
        shifted = np.roll(m1.reshape(shape), (3, 5), axis=(2, 3)).reshape(m1.shape)
        hs = demag(lat, M, shifted)
        assert rel(hs, np.roll(h1.reshape(shape), (3, 5), axis=(2, 3)).reshape(h1.shape)) <= 1e-12
    with M.Lattice(c32) as lat:
        lat.build_demag(cache)  # the cached FP64 tensor
        h32 = demag(lat, M, m1)
    assert rel(h32, h1) <= 1e-5


def test_slab_fp32_sweeps_energy_matches_fp64_evaluation(M, cache):
    c32 = M.Config.defaults(precision=32, **SLAB)
    c64 = M.Config.defaults(precision=64, **SLAB)
    with M.Lattice(c32) as lat:
        lat.build_demag(cache)
        lat.run_sweeps(800.0, 0, 0, 20)
        m = lat.get_m()
        o32 = lat.energy()
    assert o32.proposed == 20 * m.shape[1] and o32.accepted > 0
    assert np.abs(np.linalg.norm(m, axis=0) - 1.0).max() < 1e-6
    with M.Lattice(c64) as lat:
        lat.build_demag(cache)
        lat.set_m(m)
        o64 = lat.energy()
    t32 = np.array([o32.e_exchange, o32.e_dmi, o32.e_anisotropy, o32.e_zeeman, o32.e_demag])
    t64 = np.array([o64.e_exchange, o64.e_dmi, o64.e_anisotropy, o64.e_zeeman, o64.e_demag])
    assert abs(o32.e_total - o64.e_total) <= 1e-4 * abs(o64.e_total)
    assert np.abs(t32 - t64).max() <= 1e-4 * np.abs(t64).sum()
    assert np.abs(np.array(o32.m) - np.array(o64.m)).max() <= 1e-6


def test_large_film_beyond_the_warp_transforms(M, tmp_path):
    """A 1500 x 1500 periodic film (one image per side): transforms of length
    1500 = 2^2 3 5^3 have no warp-level plan and run on the general mixed-radix
    path, and in FP64 the column pass's tensor tile does not fit beside its
    line buffers, so the pass reads the tensor from global memory.  FP64
    linearity (1e-12) and the FP32 field against the FP64 field of the same
    state (1e-5).  (Sides whose transform needs more shared memory than a CTA
    has -- 2048 periodic, 600 open -- are refused at creation.)"""
    geom = dict(nx=1500, ny=1500, nz=1, dx=2e-9, dy=2e-9, dz=1e-9, pbc_x=1, pbc_y=1, pbc_z=0, cal_demag_flag=1,
                randomseed=3, sweep_engine=1)
    cache = str(tmp_path)
    with M.Lattice(M.Config.defaults(precision=64, **geom)) as lat:
        lat.build_demag(cache)
        m1 = lat.get_m().astype(np.float32).astype(np.float64)
        m2 = np.roll(m1, 7, axis=1)
        h1 = demag(lat, M, m1)
        h2 = demag(lat, M, m2)
        h12 = demag(lat, M, m1 - 0.5 * m2)
        assert rel(h12, h1 - 0.5 * h2) <= 1e-12
    with M.Lattice(M.Config.defaults(precision=32, **geom)) as lat:
        lat.build_demag(cache)
        h32 = demag(lat, M, m1)
    assert rel(h32, h1) <= 1e-5
    with pytest.raises(M.MmcError) as ei:
        M.Lattice(M.Config.defaults(precision=32, **dict(geom, nx=2048, ny=2048)))
    assert ei.value.status == M.ERR_UNSUPPORTED
