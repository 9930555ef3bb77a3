"""Batched replicas and parallel tempering (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cfgs_for(M, R, prec, **kw):
    out = []
    for r in range(R):
        base = dict(nx=32, ny=24, nz=1, pbc_x=2, pbc_y=1, pbc_z=0, precision=prec, randomseed=100 + 7 * r,
                    Bextz=0.1 + 0.05 * r, Dind=3e-3 + 1e-3 * r, Temperature_start=150.0 + 40 * r)
        base.update(kw)
        out.append(M.Config.defaults(**base))
    return out


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("geom", [dict(), dict(nx=12, ny=10, nz=3, pbc_x=0, pbc_y=0, pbc_z=0),
                                  dict(nx=15, ny=8, pbc_x=1, pbc_y=1)])
def test_batch_replicas_equal_single_runs(M, prec, geom):
    cfgs = cfgs_for(M, 3, prec, **geom)
    with M.Batch(cfgs) as b:
        b.run_sweeps(2, 0, 45)
        obs = b.energy()
        ms = [b.get_m(r) for r in range(3)]
    for r, c in enumerate(cfgs):
        with M.Lattice(c) as lat:
            lat.run_sweeps(c.Temperature_start, 2, 0, 45)
            o = lat.energy()
            assert np.array_equal(lat.get_m(), ms[r]), r
        assert o.accepted == obs[r].accepted
        assert o.e_total == pytest.approx(obs[r].e_total, rel=1e-12 if prec == 64 else 1e-6)


@pytest.mark.parametrize("prec", [32, 64])
def test_batch_row_kernel_equals_pass_kernels(M, prec):
    """Film batches run as row kernel + column pass; more CTAs than fit on the
    device at once, so bands read halo rows written by earlier waves unless the
    two copies of m and the spectrum keep them apart.  Odd sweep counts end in
    the second copy and are moved back."""
    kw = dict(nx=128, ny=128, pbc_x=2, pbc_y=2)
    rows = cfgs_for(M, 12, prec, sweep_engine=2, **kw)
    plain = cfgs_for(M, 12, prec, sweep_engine=1, **kw)
    with M.Batch(rows) as a, M.Batch(plain) as b:
        assert a.launch_shape()[5] > 0 and b.launch_shape()[5] == 0
        # a smaller lattice created later must not lower the first one's
        # shared-memory limit
        with M.Batch(cfgs_for(M, 2, prec, sweep_engine=2, nx=16, ny=8)) as small:
            small.run_sweeps(1, 0, 3)
        for s0, n in ((0, 33), (33, 64), (97, 1)):
            a.run_sweeps(1, s0, n)
            b.run_sweeps(1, s0, n)
        for r in range(12):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        ea, eb = a.energy(), b.energy()
        assert [o.accepted for o in ea] == [o.accepted for o in eb]


@pytest.mark.parametrize("geom", [dict(nx=64, ny=48, pbc_x=2, pbc_y=2), dict(nx=12, ny=10, nz=3, pbc_x=0, pbc_y=0)])
def test_batch_autotune_keeps_state_and_results(M, geom):
    """The autotuner runs sweeps with every launch shape, then restores m and
    the counters: a tuned batch continues exactly as an untuned one."""
    cfgs = cfgs_for(M, 5, 32, **geom)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        a.run_sweeps(0, 0, 5)
        b.run_sweeps(0, 0, 5)
        m0 = [a.get_m(r) for r in range(5)]
        ms, n = a.autotune(4)
        assert ms > 0 and n >= 2
        for r in range(5):
            assert np.array_equal(a.get_m(r), m0[r])
        a.run_sweeps(0, 5, 41)
        b.run_sweeps(0, 5, 41)
        for r in range(5):
            assert np.array_equal(a.get_m(r), b.get_m(r)), (r, a.launch_shape())
        assert [o.accepted for o in a.energy()] == [o.accepted for o in b.energy()]


TILE_GEOMS = [dict(nx=64, ny=64, pbc_x=1, pbc_y=1), dict(nx=96, ny=41, pbc_x=1, pbc_y=0),
              dict(nx=41, ny=23, pbc_x=0, pbc_y=0), dict(nx=12, ny=2, pbc_x=1, pbc_y=1),
              dict(nx=4, ny=1, pbc_x=1, pbc_y=1), dict(nx=20, ny=10, pbc_x=0, pbc_y=1)]


def form_ok(geom, form):
    """Eligibility of the tile (1), vector (2), staged vector (3), strip (4)
    and pipelined staged (5) forms for a two-colour film."""
    nx, ny = geom["nx"], geom["ny"]
    if form in (2, 4):
        return nx % 4 == 0
    if form in (3, 5):
        return nx % 4 == 0 and nx <= 1024
    per_ok = lambda n, p: p == 0 or (n % 32 == 0 and n >= 64)
    return per_ok(nx, geom.get("pbc_x", 2)) and per_ok(ny, geom.get("pbc_y", 1))


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("geom", TILE_GEOMS)
@pytest.mark.parametrize("form", [1, 2, 3, 4, 5])
def test_mc_forms_bitwise_equal_scalar_kernels(M, prec, geom, form):
    """Both colours in one tile launch (ring of colour-0 cells recomputed), the
    vectorised per-colour form, the same with the rows staged in shared
    memory, both colours in one launch by strips of rows (the rows next to a
    strip recomputed; m read from one copy and written to the other), or the
    staged form by persistent CTAs with the rows fetched by bulk asynchronous
    copies (a chunk of bands of several replicas per CTA), against the scalar
    per-colour form.  37 + 32 sweeps: the strip form's odd run ends in the
    second copy and is moved back."""
    if not form_ok(geom, form):
        pytest.skip("form not available for this lattice (checked in test_mc_forms_rejected_where_ineligible)")
    cfgs = cfgs_for(M, 3, prec, sweep_engine=1, **geom)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sa, sb = list(a.launch_shape()), list(b.launch_shape())
        sa[6], sb[6] = 0, form
        a.set_launch_shape(sa)
        b.set_launch_shape(sb)
        assert a.launch_shape()[6] == 0 and b.launch_shape()[6] == form
        for s0, n in ((0, 37), (37, 32)):
            a.run_sweeps(3, s0, n)
            b.run_sweeps(3, s0, n)
        for r in range(3):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert [o.accepted for o in a.energy()] == [o.accepted for o in b.energy()]


QUAD3D_GEOMS = [dict(nx=8, ny=6, nz=4, pbc_x=1, pbc_y=1, pbc_z=0), dict(nx=12, ny=5, nz=4, pbc_x=2, pbc_y=0, pbc_z=1),
                dict(nx=16, ny=8, nz=2, pbc_x=1, pbc_y=1, pbc_z=1)]


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("geom", QUAD3D_GEOMS)
def test_vector_form_on_3d_lattices(M, O, prec, geom):
    """The vectorised per-colour form with neighbour layers (3-D lattices)
    against the scalar form, and in FP64 against the oracle's decisions."""
    cfgs = cfgs_for(M, 2, prec, sweep_engine=1, **geom)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sa, sb = list(a.launch_shape()), list(b.launch_shape())
        sa[6], sb[6] = 0, 2
        a.set_launch_shape(sa)
        b.set_launch_shape(sb)
        m0 = b.get_m(0)
        for s0, n in ((0, 21), (21, 32)):
            a.run_sweeps(3, s0, n)
            b.run_sweeps(3, s0, n)
        for r in range(2):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        ob = b.energy()  # the accept counters are read once
        assert [o.accepted for o in a.energy()] == [o.accepted for o in ob]
        got = b.get_m(0)
        acc = ob[0].accepted
    if prec == 64:
        c = cfgs[0]
        with M.Lattice(c) as lat:
            k6 = lat.tensor()
        m = m0.copy()
        want = O.sweeps(c, k6, c.Temperature_start, 3, 0, 53, m, demag_mode=1)
        assert acc == want
        assert np.array_equal(got, m)


@pytest.mark.parametrize("form", [1, 2, 3, 5])
def test_mc_forms_fp64_decisions_match_oracle(M, O, form):
    c = cfgs_for(M, 1, 64, sweep_engine=1, nx=64, ny=64, pbc_x=1, pbc_y=1)[0]
    with M.Batch([c]) as b:
        s = list(b.launch_shape())
        s[6] = form
        b.set_launch_shape(s)
        m0 = b.get_m(0)
        b.run_sweeps(2, 0, 60)
        got = b.get_m(0)
        acc = b.energy()[0].accepted
        k6 = None
    with M.Lattice(c) as lat:
        k6 = lat.tensor()
    m = m0.copy()
    want_acc = O.sweeps(c, k6, c.Temperature_start, 2, 0, 60, m, demag_mode=1)
    assert acc == want_acc
    assert np.array_equal(got, m)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("geom", [dict(nx=64, ny=64, pbc_x=2, pbc_y=2), dict(nx=32, ny=128, pbc_x=1, pbc_y=1),
                                  dict(nx=16, ny=32, nz=2, pbc_x=1, pbc_y=1, pbc_z=0),
                                  dict(nx=12, ny=10, nz=3, pbc_x=0, pbc_y=0),
                                  dict(nx=40, ny=256, pbc_x=1, pbc_y=2), dict(nx=24, ny=100, pbc_x=2, pbc_y=0)])
@pytest.mark.parametrize("variant", ["inline", "lean", "lean_half_threads", "two_streams", "regs", "regs3"])
def test_transform_variants_bitwise_equal(M, prec, geom, variant):
    """The pass kernels with the warp-level transforms in line or out of line,
    the in-place column passes that read K^ from global memory (with the full
    or half thread count), and the film column pass held in registers, all
    three components per thread (k_col_reg) or one (k_col_reg3) -- y lengths
    64 and 256: ny = 256 periodic, and 100 open, its 199 padded to 256; the
    other lattices fall back to the in-place pass -- round identically."""
    cfgs = cfgs_for(M, 2, prec, sweep_engine=1, **geom)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sa, sb = list(a.launch_shape()), list(b.launch_shape())
        sa[7] = sa[8] = 0
        if variant == "inline":
            sb[7] = 1
        elif variant == "two_streams":
            sb[9] = 2
        elif variant == "regs":
            sb[8] = 2
        elif variant == "regs3":
            sb[8] = 3
        else:
            sb[8] = 1
            if variant == "lean_half_threads":
                sb[4] = max(64, sb[4] // 2)
        a.set_launch_shape(sa)
        b.set_launch_shape(sb)
        a.run_sweeps(1, 0, 29)
        b.run_sweeps(1, 0, 29)
        a.run_sweeps(1, 29, 64)  # graph replays
        b.run_sweeps(1, 29, 64)
        for r in range(2):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert [o.accepted for o in a.energy()] == [o.accepted for o in b.energy()]


def test_mc_forms_rejected_where_ineligible(M):
    # a 48-wide periodic axis is not a whole number of 32-cell tiles
    with M.Batch(cfgs_for(M, 1, 32, nx=48, ny=64, pbc_x=1, pbc_y=1)) as b:
        s = list(b.launch_shape())
        assert s[6] == 0  # one replica: the scalar form by default
        s[6] = 1
        with pytest.raises(M.MmcError):
            b.set_launch_shape(s)
    # the vector forms need nx % 4 == 0, the staged one also nx <= 1024
    with M.Batch(cfgs_for(M, 1, 32, nx=18, ny=8, pbc_x=1, pbc_y=1)) as b:
        s = list(b.launch_shape())
        assert s[6] == 0
        for form in (2, 3, 5):
            s[6] = form
            with pytest.raises(M.MmcError):
                b.set_launch_shape(s)
    with M.Batch(cfgs_for(M, 1, 32, nx=1040, ny=2, pbc_x=1, pbc_y=1)) as b:
        s = list(b.launch_shape())
        s[6] = 2
        b.set_launch_shape(s)
        for form in (3, 5, 6):
            s[6] = form
            with pytest.raises(M.MmcError):
                b.set_launch_shape(s)
    # the staged forms are for films
    with M.Batch(cfgs_for(M, 1, 32, nx=8, ny=6, nz=3, pbc_x=1, pbc_y=1, pbc_z=0)) as b:
        s = list(b.launch_shape())
        s[6] = 5
        with pytest.raises(M.MmcError):
            b.set_launch_shape(s)


def test_batch_temperatures_and_chunking(M):
    cfgs = cfgs_for(M, 4, 32)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        T = np.array([100.0, 200.0, 300.0, 400.0])
        a.set_temperatures(T)
        b.set_temperatures(T)
        a.run_sweeps(0, 0, 70)
        b.run_sweeps(0, 0, 33)
        b.run_sweeps(0, 33, 37)
        for r in range(4):
            assert np.array_equal(a.get_m(r), b.get_m(r))
        assert np.array_equal(a.temperatures(), T)


def test_parallel_tempering_first_round_matches_host_rule(M, O):
    """After one swap interval, the ladder state equals the swap rule applied on
    the host to the energies of the same states."""
    K = 6
    temps = 60.0 * (1.5 ** np.arange(K))
    cfgs = [M.Config.defaults(nx=24, ny=24, nz=1, pbc_x=1, pbc_y=1, pbc_z=0, precision=64, randomseed=11 + r)
            for r in range(K)]
    interval = 10
    with M.Batch(cfgs) as plain:
        plain.set_temperatures(temps)
        plain.run_sweeps(0, 0, interval)
        E = np.array([o.e_total for o in plain.energy()])
    with M.Batch(cfgs) as pt:
        pt.set_ladders(np.arange(K)[None, :], temps[None, :], interval, seed=1234)
        pt.run_sweeps(0, 0, interval)
        rep, cnt = pt.ladder_state()
        Tnow = pt.temperatures()
    kB = 1.3806488e-23
    at = list(range(K))
    acc = 0
    for k in range(0, K - 1, 2):  # round 0: even pairs
        a, b = at[k], at[k + 1]
        delta = (1 / (kB * temps[k]) - 1 / (kB * temps[k + 1])) * (E[a] - E[b])
        r = O.philox([0, 0, k, 2], [1234, 0])[0]
        u = (r + 0.5) * 2.0 ** -32
        if delta >= 0 or u < np.exp(delta):
            at[k], at[k + 1] = b, a
            acc += 1
    assert list(rep[0]) == at
    assert int(cnt[0]) == K // 2 and int(cnt[1]) == acc
    for k in range(K):
        assert Tnow[at[k]] == temps[k]


def test_parallel_tempering_invariants(M):
    nl, K = 2, 4
    cfgs = [M.Config.defaults(nx=16, ny=16, nz=1, pbc_x=1, pbc_y=1, pbc_z=0, precision=32, randomseed=r + 1,
                              Bextz=0.2 if r < K else 0.4) for r in range(nl * K)]
    temps = np.array([[50.0, 90.0, 160.0, 290.0]] * nl)
    reps = np.arange(nl * K).reshape(nl, K)
    with M.Batch(cfgs) as b:
        b.set_ladders(reps, temps, 10, seed=7)
        b.run_sweeps(0, 0, 200)
        rep, cnt = b.ladder_state()
        T = b.temperatures()
    rounds = 20
    assert int(cnt[0]) == nl * (rounds // 2 * 2 + rounds // 2 * 1)
    assert 0 < int(cnt[1]) <= int(cnt[0])
    for l in range(nl):
        assert sorted(rep[l]) == sorted(reps[l])  # swaps stay inside a ladder
        for k in range(K):
            assert T[rep[l, k]] == temps[l, k]


def test_batch_rejects_mixed_geometry(M):
    a = M.Config.defaults(nx=16, ny=16)
    b = M.Config.defaults(nx=16, ny=8)
    with pytest.raises(M.MmcError):
        M.Batch([a, b])


@pytest.mark.parametrize("streams", [2, 3, 4])
def test_streams_with_tempering_and_odd_batch(M, streams):
    """Replica parts on several streams for a batch of odd size with
    parallel-tempering ladders: the swap pass runs after every part, results
    equal the one-stream batch."""
    cfgs = cfgs_for(M, 5, 32, sweep_engine=1, nx=32, ny=32, pbc_x=1, pbc_y=1)
    temps = np.array([[60.0, 100.0, 170.0, 290.0, 500.0]])
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        s = list(b.launch_shape())
        s[9] = streams
        b.set_launch_shape(s)
        for x in (a, b):
            x.set_ladders(np.arange(5).reshape(1, 5), temps, 10, 3)
            x.run_sweeps(0, 0, 95)
        for r in range(5):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert np.array_equal(a.temperatures(), b.temperatures())


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("geom", [dict(nx=1024, ny=6, pbc_x=1, pbc_y=1), dict(nx=512, ny=9, pbc_x=1, pbc_y=0),
                                  dict(nx=8, ny=300, pbc_x=0, pbc_y=1)])
def test_pipelined_form_wide_and_tall_films(M, prec, geom):
    """The pipelined staged form where its buffers are largest (one row per
    band at nx = 1024: 96 KB per buffer in FP64) or hold many rows (nx = 8:
    bands of 128 rows), with open and periodic y edges and replicas spread
    over two streams, against the scalar per-colour form."""
    cfgs = cfgs_for(M, 5, prec, sweep_engine=1, **geom)
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sa, sb = list(a.launch_shape()), list(b.launch_shape())
        sa[6], sb[6] = 0, 5
        sb[9] = 2
        a.set_launch_shape(sa)
        b.set_launch_shape(sb)
        for s0, n in ((0, 7), (7, 32)):
            a.run_sweeps(2, s0, n)
            b.run_sweeps(2, s0, n)
        for r in range(5):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert [o.accepted for o in a.energy()] == [o.accepted for o in b.energy()]


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("streams", [1, 3])
def test_strip_form_with_streams_tempering_and_profile(M, prec, streams):
    """The strip form (form 4: both colours in one launch, m alternating
    between two copies) on replica parts on several streams, with
    parallel-tempering ladders swapping every 7 sweeps (odd graphs end in the
    second copy), and through the profiling path with an odd sweep count:
    results equal the scalar one-stream batch."""
    cfgs = cfgs_for(M, 5, prec, sweep_engine=1, nx=32, ny=32, pbc_x=1, pbc_y=1)
    temps = np.array([[60.0, 100.0, 170.0, 290.0, 500.0]])
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        sa, sb = list(a.launch_shape()), list(b.launch_shape())
        sa[6], sa[9] = 0, 1
        sb[6], sb[9] = 4, streams
        a.set_launch_shape(sa)
        b.set_launch_shape(sb)
        assert b.launch_shape()[6] == 4
        for x in (a, b):
            x.set_ladders(np.arange(5).reshape(1, 5), temps, 7, 3)
            x.run_sweeps(0, 0, 95)
        for r in range(5):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert np.array_equal(a.temperatures(), b.temperatures())
        a.profile_sweeps(1, 0, 5)
        b.profile_sweeps(1, 0, 5)
        for r in range(5):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert [o.accepted for o in a.energy()] == [o.accepted for o in b.energy()]


def test_strip_form_rejected_where_ineligible(M):
    """The strip form needs a two-colour film with nx a multiple of 4."""
    for geom in (dict(nx=41, ny=23, pbc_x=0, pbc_y=0), dict(nx=15, ny=8, pbc_x=1, pbc_y=1),
                 dict(nx=8, ny=6, nz=3, pbc_x=1, pbc_y=1, pbc_z=0)):
        with M.Batch(cfgs_for(M, 2, 32, sweep_engine=1, **geom)) as b:
            s = list(b.launch_shape())
            s[6] = 4
            with pytest.raises(M.MmcError):
                b.set_launch_shape(s)


def test_parallel_tempering_fp32_swap_energies(M, O):
    """FP32 replicas swap on energies summed from FP32 per-cell terms
    (k_energy_lean): the first round's decisions equal the host rule applied
    to the FP64-per-cell energies of the same states wherever the decision is
    not a near-tie (|delta - log u| above the ~1e-6 relative energy difference
    times |E| / kT)."""
    K = 8
    temps = 80.0 * (1.35 ** np.arange(K))
    cfgs = [M.Config.defaults(nx=64, ny=64, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=32, randomseed=21 + r)
            for r in range(K)]
    interval = 10
    with M.Batch(cfgs) as plain:
        plain.set_temperatures(temps)
        plain.run_sweeps(0, 0, interval)
        E = np.array([o.e_total for o in plain.energy()])
    with M.Batch(cfgs) as pt:
        pt.set_ladders(np.arange(K)[None, :], temps[None, :], interval, seed=77)
        pt.run_sweeps(0, 0, interval)
        rep, cnt = pt.ladder_state()
    kB = 1.3806488e-23
    at = list(range(K))
    checked = 0
    for k in range(0, K - 1, 2):
        a, b = at[k], at[k + 1]
        delta = (1 / (kB * temps[k]) - 1 / (kB * temps[k + 1])) * (E[a] - E[b])
        r = O.philox([0, 0, k, 2], [77, 0])[0]
        u = (r + 0.5) * 2.0 ** -32
        margin = abs(min(delta, 0.0) - np.log(u))
        tol = 1e-5 * abs(1 / (kB * temps[k]) - 1 / (kB * temps[k + 1])) * (abs(E[a]) + abs(E[b]))
        swapped = rep[0][k] == b
        if margin > tol:
            assert swapped == (delta >= 0 or u < np.exp(delta)), k
            checked += 1
    assert checked >= 3 and int(cnt[0]) == K // 2


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("form", [2, 4, 5])
def test_tempering_swap_fused_into_next_sweep(M, prec, form):
    """One call of 95 sweeps with swaps every 10 (graphs whose first sweep
    makes the previous interval's swap from the demag field it computes
    anyway) against the same sweeps in calls of 7 (separate swap passes before
    direct sweeps): equal states, temperatures and swap counts, with the
    vectorised (2) and strip (4) Metropolis forms."""
    cfgs = cfgs_for(M, 6, prec, sweep_engine=1, nx=32, ny=32, pbc_x=1, pbc_y=1)
    temps = np.array([[50.0, 80.0, 130.0, 210.0, 340.0, 550.0]])
    with M.Batch(cfgs) as a, M.Batch(cfgs) as b:
        for x in (a, b):
            s = list(x.launch_shape())
            s[6] = form
            x.set_launch_shape(s)
            x.set_ladders(np.arange(6).reshape(1, 6), temps, 10, 5)
        a.run_sweeps(0, 0, 95)
        s0 = 0
        while s0 < 95:
            k = min(7, 95 - s0)
            b.run_sweeps(0, s0, k)
            s0 += k
        for r in range(6):
            assert np.array_equal(a.get_m(r), b.get_m(r)), r
        assert np.array_equal(a.temperatures(), b.temperatures())
        ra, ca = a.ladder_state()
        rb, cb = b.ladder_state()
        # 9 rounds: 5 even ones with 3 pairs, 4 odd ones with 2
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb) and int(ca[0]) == 5 * 3 + 4 * 2
