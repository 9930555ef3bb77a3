"""bench.py host logic that needs no GPU: the roofline's DRAM-traffic lookup
in the committed ncu summary (replica-tagged lines, scaling of a capture at
another replica count) and the launch count of a timed step."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _lines():
    out = []
    with open(os.path.join(ROOT, "profiles", "batched_256x256_kernels.md")) as f:
        for line in f:
            parts = line.strip().split()
            if parts and parts[0] == "dram_bytes_per_launch":
                out.append(parts)
    return out


def test_traffic_lines_parse():
    lines = _lines()
    assert lines, "no traffic lines in the ncu summary"
    for p in lines:
        assert len(p) in (4, 5)
        assert len(p[2].rstrip(":").split(",")) == 10
        assert float(p[-1]) > 0
        if len(p) == 5:
            assert p[3].startswith("r") and int(p[3].rstrip(":")[1:]) > 0


def test_traffic_lookup_prefers_replica_count_and_shape():
    shape = [4, 128, 8, 64, 384, 0, 2, 1, 3, 1]
    v64, note64 = bench.ncu_traffic("k_mc_quad", shape, 64)
    v32, note32 = bench.ncu_traffic("k_mc_quad", shape, 32)
    assert "64 replicas" in note64 and "scaled" not in note64
    assert "32 replicas" in note32 and "scaled" not in note32
    # a launch's cold-cache traffic is one pass over its replicas' data
    assert 1.9 < v64 / v32 < 2.1
    # another count is scaled from the nearest capture and says so
    v16, note16 = bench.ncu_traffic("k_mc_quad", shape, 16)
    assert "scaled to 16 replicas" in note16
    assert abs(v16 - v32 / 2) < 1e-6 * v32 or abs(v16 - v64 / 4) < 1e-6 * v64
    assert bench.ncu_traffic("k_no_such_kernel", shape, 64) == (None, None)


def test_launches_per_step():
    S, R = 10000, 64
    # pass kernels, vectorised Metropolis (two launches per sweep), 2 streams:
    # 5 launches per sweep and part inside the graphs, one counter advance per
    # graph and one after the 16 sweeps left over
    shape = [4, 128, 4, 64, 192, 0, 2, 1, 2, 2]
    graphs, rem = divmod(S, 32)
    assert bench.launches_per_step(S, shape, R) == graphs * 32 * 5 * 2 + rem * 5 + graphs + 1
    # both colours in one launch (tile, strip): 4 launches per sweep
    for form in (1, 4):
        one = list(shape)
        one[6] = form
        assert bench.launches_per_step(S, one, R) == graphs * 32 * 4 * 2 + rem * 4 + graphs + 1
    # the row kernel: two launches per sweep, one part
    rows = [4, 128, 4, 64, 192, 4, 2, 1, 2, 2]
    assert bench.launches_per_step(S, rows, R) == graphs * 32 * 2 + rem * 2 + graphs + 1
