"""The multi-GPU host logic of bench.py on CPU: two gloo ranks (replicas only,
no data-path collective): the max-over-ranks timing, the barrier, disjoint
replica seeds, and the reference arm doing no work on ranks other than 0."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist, r, local, w = bench.dist_setup()
    bench.barrier(dist)
    t = bench.reduce_max(dist, 1.0 + rank)
    seeds = bench.replica_seeds(rank, 4)
    # the reference arm returns at once on ranks other than 0
    ref_done = None
    if rank != 0:
        class A:
            ref_seconds = 0.0
        bench.run_reference(A())
        ref_done = True
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((rank, r, w, t, seeds, ref_done))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, rr0, w0, t0, s0, _), (r1, rr1, w1, t1, s1, ref1) = out
    assert (rr0, rr1, w0, w1) == (0, 1, 2, 2)
    assert t0 == t1 == 2.0
    assert not set(s0) & set(s1) and s0[0] == 256
    assert ref1 is True


def test_launch_count_of_a_step():
    """bench.py's gpu_launches: per sweep the 5 pass kernels once per replica
    part inside the 32-sweep graphs and on one stream for the left-over
    sweeps, 2 for the row path, 4 with the tile form; one counter advance per
    graph and after the left-over sweeps."""
    sys.path.insert(0, ROOT)
    import bench

    shape = [4, 128, 8, 64, 384, 0, 2, 1, 1, 2]
    assert bench.launches_per_step(10000, shape, 32) == 312 * 32 * 5 * 2 + 16 * 5 + 312 + 1
    assert bench.launches_per_step(64, shape, 1) == 64 * 5 + 2  # one replica: one part
    rows = [4, 128, 8, 8, 384, 4, 2, 1, 1, 3]
    assert bench.launches_per_step(40, rows, 32) == 40 * 2 + 2
    tile = [4, 128, 8, 8, 384, 0, 1, 1, 1, 1]
    assert bench.launches_per_step(32, tile, 8) == 32 * 4 + 1
