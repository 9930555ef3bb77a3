"""Replica farms: batches of different lattice sizes advanced in one call, and
the parallel-tempering layout of the batched workload (4 ladders of 16
temperatures over 40-1400 K, swaps every 10 sweeps, square films of side
64..256 with per-ladder field and DMI)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MATERIAL = dict(nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, ms=1.6e6, Aex=16e-12, Dind=6e-3, Ku1=2e6, anisUx=0, anisUy=0,
                anisUz=1, Bextx=0, Bexty=0, Bextz=0.3, pbc_x=2, pbc_y=2, pbc_z=0)


def ladder_batch(M, side, nladders, per, seed0, bz, dind, prec=32, temps=(40.0, 1400.0)):
    T = np.geomspace(temps[0], temps[1], per)
    cfgs = [M.Config.defaults(precision=prec, nx=side, ny=side, randomseed=seed0 + k,
                              **dict(MATERIAL, Bextz=bz[k // per], Dind=dind[k // per]))
            for k in range(nladders * per)]
    b = M.Batch(cfgs)
    reps = np.arange(nladders * per, dtype=np.int32).reshape(nladders, per)
    b.set_ladders(reps, np.tile(T, (nladders, 1)), 10, 1234 + seed0)
    return b


def test_farm_equals_separate_batches(M):
    def make():
        return [ladder_batch(M, 64, 1, 4, 1, [0.2], [4e-3]), ladder_batch(M, 96, 2, 3, 11, [0.3, 0.4], [5e-3, 3e-3])]

    farm_b = make()
    solo_b = make()
    try:
        with M.Farm(farm_b) as f:
            f.run_sweeps(0, 0, 45)
            f.run_sweeps(1, 0, 17)
            assert f.last_run_ms() > 0
        for b in solo_b:
            b.run_sweeps(0, 0, 45)
            b.run_sweeps(1, 0, 17)
        for a, b in zip(farm_b, solo_b):
            for r in range(a.R):
                assert np.array_equal(a.get_m(r), b.get_m(r))
            assert np.array_equal(a.temperatures(), b.temperatures())
            ra, ca = a.ladder_state()
            rb, cb = b.ladder_state()
            assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
    finally:
        for b in farm_b + solo_b:
            b.close()


def test_pt_farm_layout(M):
    """The batched parallel-tempering workload at reduced sweeps: seeds 1..64,
    each ladder draws its side, B_z and DMI; ladders of one side share a
    batch; after the run every ladder still holds its 16 temperatures."""
    rng = np.random.default_rng(2024)
    sides = rng.choice([64, 96, 128, 192, 256], size=4)
    bz = rng.uniform(0.1, 0.5, size=4)
    dind = rng.uniform(3e-3, 6e-3, size=4)
    batches = []
    seed = 1
    for side in sorted(set(sides.tolist())):
        ls = [i for i in range(4) if sides[i] == side]
        batches.append(ladder_batch(M, int(side), len(ls), 16, seed, bz[ls], dind[ls]))
        seed += 16 * len(ls)
    try:
        for b in batches:
            b.autotune(4)
        with M.Farm(batches) as f:
            f.run_sweeps(0, 0, 200)
        T = np.geomspace(40.0, 1400.0, 16)
        for b in batches:
            reps, counts = b.ladder_state()
            temps = b.temperatures()
            for ladder in reps:
                assert np.allclose(np.sort(temps[ladder]), T, rtol=1e-12)
            assert counts[0] > 0 and 0 < counts[1] <= counts[0]
    finally:
        for b in batches:
            b.close()
