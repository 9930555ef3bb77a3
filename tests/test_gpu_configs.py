"""Parity at the benchmark configurations themselves (GPU).

Workloads, with the material of the 64x64x1 / 256x256x1 anneal: dx = dy = 1 nm,
dz = 0.8 nm, Ms = 1.6e6 A/m, Aex = 16e-12 J/m, Dind = 6e-3 J/m^2, Ku1 = 2e6 J/m^3
along z, Bext = (0, 0, 0.3) T, 20 periodic images in x and y, open z, demag on,
T from 1400 K down by x0.90 per stage.

- FP64 accept/reject decisions bit-identical to the oracle's for 100 sweeps
  at 64x64x1 (seed 256) and at 256x256x1, at the first stage's temperature
  and at the last stage's;
- the batched FP32 vectorised Metropolis form at 256x256x1 (64 replicas, the
  benchmark's batch) against batched FP64 from the same states;
- the stage loop's energy.txt lines and final state against the oracle's.

The oracle gets the GPU's tensor as input; that tensor equals the oracle's own
bit for bit and the reference's ktensorCPU to its rounding (test_gpu_parity,
test_gpu_ref_pin)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MATERIAL = dict(dx=1e-9, dy=1e-9, dz=0.8e-9, ms=1.6e6, Aex=16e-12, Dind=6e-3, Ku1=2e6, anisUx=0, anisUy=0,
                anisUz=1, Bextx=0, Bexty=0, Bextz=0.3, pbc_x=20, pbc_y=20, pbc_z=0, cal_demag_flag=1,
                Temperature_start=1400.0, Temperature_end=40.0, Temperature_step=0.9, Temperature_use_exp=1,
                rand_block_size=40)
T_FIRST, STAGE_LAST = 1400.0, 33
T_LAST = 1400.0 * 0.9 ** STAGE_LAST  # 43.7 K, the last stage above 40 K


@pytest.fixture(scope="module")
def cache(tmp_path_factory):
    return str(tmp_path_factory.mktemp("tensor_cache"))


def config(M, side, prec, seed, **kw):
    return M.Config.defaults(nx=side, ny=side, nz=1, precision=prec, randomseed=seed, **dict(MATERIAL, **kw))


@pytest.mark.parametrize("side,seed", [(64, 256), (256, 256)])
@pytest.mark.parametrize("T,stage", [(T_FIRST, 0), (T_LAST, STAGE_LAST)])
def test_fp64_decisions_bitwise_at_benchmark_configs(M, O, cache, side, seed, T, stage):
    c = config(M, side, 64, seed)
    with M.Lattice(c) as lat:
        lat.build_demag(cache)
        k = lat.tensor()
        m0 = lat.get_m()
        lat.run_sweeps(T, stage, 0, 100)
        m_gpu = lat.get_m()
        o = lat.energy()
    assert np.array_equal(m0, O.init_random(c, seed))
    m = m0.copy()
    acc = O.sweeps(c, k, T, stage, 0, 100, m, demag_mode=1)
    assert o.proposed == 100 * side * side
    assert o.accepted == acc
    assert np.array_equal(m_gpu, m)
    # the decisions are not trivial: some rejected, most at the low temperature
    assert 0 < acc < o.proposed


def test_batched_fp32_vector_form_tracks_fp64_at_256(M, cache):
    """64 replicas of 256x256x1 (seeds 256..319) through the vectorised FP32
    Metropolis form, against 64 FP64 replicas from the same FP32-representable
    states: both use the same Philox stream, so they make the same decisions
    until a near-tie; after 3 sweeps nearly every spin agrees to FP32 rounding
    and the energies agree to 1e-4 relative."""
    R = 64
    c32 = [config(M, 256, 32, 256 + r) for r in range(R)]
    c64 = [config(M, 256, 64, 256 + r) for r in range(R)]
    with M.Batch(c32) as a, M.Batch(c64) as b:
        a.build_demag(cache)
        b.build_demag(cache)
        # pass kernels (4-row x passes of 128 threads, 8-column passes of 384
        # threads), the vectorised Metropolis form, one stream
        a.set_launch_shape([4, 128, 8, 64, 384, 0, 2, 1, 1, 1])
        assert a.launch_shape()[6] == 2
        for r in range(R):
            b.set_m(r, a.get_m(r))
        T = np.full(R, 300.0)
        a.set_temperatures(T)
        b.set_temperatures(T)
        a.run_sweeps(0, 0, 3)
        b.run_sweeps(0, 0, 3)
        agree = np.mean([np.all(np.abs(a.get_m(r) - b.get_m(r)) < 1e-5, axis=0).mean() for r in range(R)])
        ea, eb = a.energy(), b.energy()
    assert agree > 0.99, agree
    rel_e = max(abs(x.e_total - y.e_total) / abs(y.e_total) for x, y in zip(ea, eb))
    assert rel_e < 1e-4, rel_e


def test_energy_txt_and_final_state_match_oracle(M, O, tmp_path):
    """The FP64 stage loop (mmc_run_anneal) on a 16x16 film with 2 images:
    every energy.txt line "%f %ld %g" equals the oracle's temperature, sweep
    and total energy printed the same way, and the final state equals the
    oracle's after the same stages, bit for bit."""
    c = M.Config.defaults(nx=16, ny=16, nz=1, precision=64, randomseed=5,
                          **dict(MATERIAL, pbc_x=2, pbc_y=2, Temperature_start=300.0, Temperature_end=200.0,
                                 circle_per_stage=20, energy_output_period=10, ms_output_period=1000,
                                 terminal_output_period=1000))
    out = tmp_path / "run.output"
    out.mkdir()
    with M.Lattice(c) as lat:
        lat.build_demag()
        k = lat.tensor()
        m0 = lat.get_m()
        lat.run_anneal(out)
        m_end = lat.get_m()
    lines = (out / "energy.txt").read_text().splitlines()
    m = m0.copy()
    want, T, stage = [], 300.0, 0
    while T > 200.0:
        for s0 in (0, 10):
            e = O.energy(c, m, O.demag_fft(c, k, m))
            want.append("%f %d %g" % (T, s0, e[:5].sum()))
            O.sweeps(c, k, T, stage, s0, 10, m, demag_mode=1)
        T *= 0.9
        stage += 1
    assert stage == 4
    assert lines == want
    assert np.array_equal(m_end, m)
