"""The GPU path against the reference's own outputs (tests/golden/ref_demag_golden.npz,
generated from the reference's ktensorCPU and calHexchangeKernel compiled
unmodified; tests/golden/make_ref_golden.py).

Tolerances (SHARED_TOL, FIELD_TOL of test_ref_pin): the FP64 tensor against
ktensorCPU within the rounding of its 64-term sums (the GPU evaluates
asinh/atan/log with its own functions, within 1 ulp of the C library's,
amplified by the sums' cancellation for far images: 1e-14 .. 5e-11 of max|K|
for few images, 1e-4 at 64x64x1 with 20 images, where the reference's own
sums are 2.6e-5 off the exact tensor); the demag field within that tensor
difference summed over the lattice (1e-12 .. 1e-3), and in FP32 within the
larger of that and 1e-5."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_demag_golden.npz")
from test_ref_pin import FIELD_TOL, SHARED_TOL  # noqa: E402


@pytest.fixture(scope="module")
def G():
    z = np.load(GOLDEN)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def _cfg(M, G, case, precision):
    c = G["meta"]["cases"][case]
    return M.Config.defaults(nx=c["nx"], ny=c["ny"], nz=c["nz"], dx=c["dx"], dy=c["dy"], dz=c["dz"],
                             pbc_x=c["pbc"][0], pbc_y=c["pbc"][1], pbc_z=c["pbc"][2], use_reference_pi=1,
                             precision=precision, cal_demag_flag=1, ms=1.6e6)


CASES = ["g0_3x2x2_open", "g1_4x4x1_pbc1", "g2_3x2x1_mixed", "g3_2x2x3_mixed", "slab6x5x4_open",
         "film8x8x3_pbc2", "cfg0_64x64x1_pbc20"]


@pytest.mark.parametrize("case", CASES)
def test_gpu_tensor_vs_reference_ktensorcpu(M, G, case):
    with M.Lattice(_cfg(M, G, case, 64)) as lat:
        lat.build_demag()
        k = lat.tensor()
    want = G["K_" + case]
    assert k.shape == want.shape
    assert np.abs(k - want).max() <= SHARED_TOL[case] * np.abs(want).max()


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("case", ["slab6x5x4_open", "film8x8x3_pbc2", "cfg0_64x64x1_pbc20"])
def test_gpu_demag_field_vs_reference_pipeline(M, G, case, prec):
    """h = K * m on the GPU against the field formed with the reference's tensor
    and product; m is the seeded initial state (its hash is in the fixture)."""
    c = _cfg(M, G, case, prec)
    seed = G["meta"]["fields"][case]
    with M.Lattice(c) as lat:
        lat.init_random(seed)
        m = lat.get_m()
        lat.build_demag()
        lat.compute_demag()
        h = lat.field(M.TERM_DEMAG) / c.ms
    if prec == 64:
        assert hashlib.sha256(m.tobytes()).hexdigest() == G["meta"]["m_sha256"][case]
        want = G["H64_" + case]
        tol = FIELD_TOL[case]
    else:
        want = G["H32_" + case].astype(np.float64)
        tol = max(1e-5, FIELD_TOL[case])
    assert np.abs(h - want).max() <= tol * np.abs(want).max()
