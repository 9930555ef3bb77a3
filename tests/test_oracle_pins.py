"""Pins the CPU oracle: its elementary functions against mpmath, Philox against the
Random123 known-answer vectors, and the Newell tensor against the 60-digit golden
evaluation of the reference's formulas (tests/golden/newell_golden.json)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Random123 known-answer vectors for philox4x32 with 10 rounds: (counter, key, result).
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_kat(O, ctr, key, want):
    assert list(O.philox(ctr, key)) == want


@pytest.mark.parametrize("fn", ["log", "asinh", "atan", "exp", "sinpi", "cospi"])
def test_elementary_functions_vs_mpmath(O, fn):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 120
    rng = np.random.default_rng(7)
    if fn == "log":
        xs = np.concatenate([10 ** rng.uniform(-300, 300, 400), rng.uniform(0.5, 2, 200), [5e-324, 1.0]])
        ref = mp.log
    elif fn in ("asinh", "atan"):
        xs = np.concatenate([10 ** rng.uniform(-30, 250, 300) * rng.choice([-1, 1], 300),
                             rng.uniform(-3, 3, 300), [0.0, 7 / 16, 11 / 16, 19 / 16, 39 / 16, 2.0]])
        ref = mp.asinh if fn == "asinh" else mp.atan
    elif fn == "exp":
        xs = np.concatenate([rng.uniform(-700, 700, 500), rng.uniform(-1, 1, 100), [0.0]])
        ref = mp.exp
    else:
        xs = np.concatenate([rng.uniform(0, 2, 500), [0.0, 0.25, 0.5, 1.0, 1.5]])
        ref = mp.sinpi if fn == "sinpi" else mp.cospi
    got = O.math(fn, xs)
    want = np.array([float(ref(mp.mpf(float(x)))) for x in xs])
    if fn in ("sinpi", "cospi"):
        err = np.abs(got - want)  # absolute, values in [-1, 1]
        assert err.max() <= 2.3e-16
    else:
        err = np.abs(got - want) / np.maximum(np.abs(want), 1e-300)
        assert err.max() <= 4.5e-16, (fn, err.max(), xs[np.argmax(err)])


def test_exp_underflow_and_sign(O):
    assert O.math("exp", np.array([-800.0]))[0] == 0.0
    assert O.math("asinh", np.array([-3.0]))[0] == -O.math("asinh", np.array([3.0]))[0]
    assert O.math("atan", np.array([-1e300]))[0] == -O.math("atan", np.array([1e300]))[0]


def _golden():
    with open(os.path.join(GOLDEN, "newell_golden.json")) as f:
        return json.load(f)


def test_newell_fg_vs_golden(O):
    G = _golden()
    for p in G["fg"]:
        f, g = O.newell_f(*p["x"]), O.newell_g(*p["x"])
        # f and g themselves cancel for some arguments; the golden is 60 digits
        scale = max(abs(v) for v in p["x"]) ** 3 + 1e-60
        assert abs(f - p["f"]) <= 1e-14 * scale, p
        assert abs(g - p["g"]) <= 1e-14 * scale, p


@pytest.mark.parametrize("case", range(4))
def test_newell_tensor_vs_golden(M, O, case):
    c = _golden()["tensors"][case]
    cfg = M.Config.defaults(nx=c["nx"], ny=c["ny"], nz=c["nz"], dx=c["dx"], dy=c["dy"], dz=c["dz"],
                            pbc_x=c["pbc"][0], pbc_y=c["pbc"][1], pbc_z=c["pbc"][2])
    assert list(O.padded_dims(cfg)) == c["padded"]
    k = O.tensor(cfg)
    K = np.array(c["K"])
    # The 64-term sum cancels catastrophically: the FP64 result of terms of size
    # ~r^3 d^3 keeps ~1e-13 of the O(1) tensor for these few-cell offsets.
    np.testing.assert_allclose(k, K, rtol=0, atol=5e-13)


def test_self_tensor_identities(M, O):
    # single cube: N = diag(1/3), K = -N, trace -1
    cfg = M.Config.defaults(nx=1, ny=1, nz=1, dx=1e-9, dy=1e-9, dz=1e-9, pbc_x=0, pbc_y=0, pbc_z=0)
    k = O.tensor(cfg)[:, 0]
    np.testing.assert_allclose(k, [-1 / 3, 0, 0, -1 / 3, 0, -1 / 3], atol=1e-15)
    # flat prism: trace still -1, Kzz most negative
    cfg = M.Config.defaults(nx=1, ny=1, nz=1, dx=2e-9, dy=1e-9, dz=0.5e-9, pbc_x=0, pbc_y=0, pbc_z=0)
    k = O.tensor(cfg)[:, 0]
    assert abs(k[0] + k[3] + k[5] + 1) < 1e-14
    assert k[5] < k[3] < k[0] < 0
    # reference pi constant changes the tensor by ~3e-12 relative only
    k_ref = O.tensor(cfg.copy(use_reference_pi=1))[:, 0]
    np.testing.assert_allclose(k_ref, k, rtol=1e-11)
    assert np.any(k_ref != k)


def test_thin_film_sum_rule(M, O):
    # A periodic thin film: sum over all offsets of K_zz tends to -1 (uniform m_z
    # gives H_d = -Ms z) and the in-plane sums to 0 as the image count grows.
    cfg = M.Config.defaults(nx=8, ny=8, nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, pbc_x=6, pbc_y=6, pbc_z=0)
    k = O.tensor(cfg)
    # finite plate of (2P+1) n = 104 cells per side and 0.8 nm thickness:
    # 1 - N_zz and N_xx are O(t/L) ~ 1e-2
    assert abs(k[5].sum() + 1) < 1.5e-2
    assert abs(k[0].sum()) < 1e-2 and abs(k[3].sum()) < 1e-2
    assert abs(k[0].sum() + k[3].sum() + k[5].sum() + 1) < 1e-9
    # K_xy sums to the unpaired far image at the even n/2 plane (r = 52 cells)
    assert abs(k[1].sum()) < 1e-6


def test_tensor_symmetry(M, O):
    cfg = M.Config.defaults(nx=5, ny=4, nz=2, dx=1e-9, dy=1.2e-9, dz=0.7e-9, pbc_x=0, pbc_y=0, pbc_z=0)
    nxp, nyp, nzp = O.padded_dims(cfg)
    k = O.tensor(cfg).reshape(6, nzp, nyp, nxp)
    # diagonal components even, xy odd in x and y
    flip_x = k[..., (-np.arange(nxp)) % nxp]
    np.testing.assert_allclose(flip_x[0], k[0], atol=1e-13)
    np.testing.assert_allclose(flip_x[1], -k[1], atol=1e-13)
    np.testing.assert_allclose(flip_x[2], -k[2], atol=1e-13)
    np.testing.assert_allclose(flip_x[4], k[4], atol=1e-13)


def test_far_field_expansion_against_60_digit_sums(O):
    """The far-field form of the 64-term sums (csrc/newell_far.h) against
    60-digit evaluations: O((d/r)^8) truncation, so < 1e-9 of the largest
    component at 12 cells and < 1e-12 beyond 30; the FP64 64-term sum itself
    is worse beyond ~20 cells (cancellation)."""
    data = json.load(open(os.path.join(GOLDEN, "newell_far_golden.json")))
    for case in data["cases"]:
        ix, iy, iz = case["cell"]
        dx, dy, dz = case["d"]
        want = np.array(case["raw"])
        got = O.newell_far(ix * dx, iy * dy, iz * dz, dx, dy, dz)
        r = np.sqrt((ix * dx) ** 2 + (iy * dy) ** 2 + (iz * dz) ** 2) / max(dx, dy, dz)
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err < (1e-9 if r < 20 else 2e-11 if r < 30 else 1e-12), (case["cell"], r, err)
        if r > 60:
            exact64 = O.newell_raw(ix, iy, iz, dx, dy, dz)
            assert np.abs(exact64 - want).max() / np.abs(want).max() > 100 * err


def test_far_radius_tensor_matches_exact_tensor(O, M):
    """A tensor with the far-field switch at 12 cells agrees with the exact one
    to the exact sum's own rounding, and equals it where no image is far."""
    c0 = M.Config.defaults(nx=16, ny=12, nz=1, pbc_x=2, pbc_y=1, pbc_z=0, precision=64)
    c1 = M.Config.defaults(nx=16, ny=12, nz=1, pbc_x=2, pbc_y=1, pbc_z=0, precision=64, tensor_far_radius=12)
    k0, k1 = O.tensor(c0), O.tensor(c1)
    assert np.abs(k1 - k0).max() <= 1e-9 * np.abs(k0).max()
    assert not np.array_equal(k0, k1)
