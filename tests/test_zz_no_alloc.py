"""mmc_demag_apply_static: the demag field with its spectrum in the library's
static device array, checked against mmc_demag_apply with caller scratch.

Collected last (file name) so that it runs both alone in a fresh process and
after every other test has used the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEOMS = [
    dict(nx=64, ny=48, nz=1, pbc_x=2, pbc_y=2, pbc_z=0, precision=32),
    dict(nx=20, ny=12, nz=2, pbc_x=1, pbc_y=0, pbc_z=0, precision=64),
    dict(nx=15, ny=9, nz=3, pbc_x=0, pbc_y=0, pbc_z=0, precision=32),
]


@pytest.mark.parametrize("geom", GEOMS)
def test_static_scratch_matches_caller_scratch(M, geom):
    torch = pytest.importorskip("torch")
    c = M.Config.defaults(**geom)
    dt = torch.float32 if geom["precision"] == 32 else torch.float64
    tol = 1e-6 if geom["precision"] == 32 else 1e-12
    dev = torch.device("cuda:0")
    with M.Lattice(c) as lat:
        lat.build_demag()
        m = torch.tensor(lat.get_m(), dtype=dt, device=dev).contiguous()
        want = torch.zeros_like(m)
        nb = lat.demag_scratch_bytes()
        scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        lat.demag_apply(m.data_ptr(), want.data_ptr(), scratch.data_ptr(), nb, None)
        torch.cuda.synchronize()
        ref = want.cpu().numpy().astype(np.float64)
        scale = np.abs(ref).max()
        assert scale > 0
        outs = [torch.full_like(m, float("nan")) for _ in range(3)]
        torch.cuda.synchronize()
        lat.demag_apply_static(m.data_ptr(), outs[0].data_ptr(), None)  # warm: module and array looked up
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        for got in outs[1:]:  # two calls in a row share the array and allocate nothing
            lat.demag_apply_static(m.data_ptr(), got.data_ptr(), None)
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info(dev)[0] == free0
        for got in outs:
            g = got.cpu().numpy().astype(np.float64)
            assert np.abs(g - ref).max() <= tol * scale


def test_static_scratch_limits(M):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    # a lattice whose spectrum is larger than the array is rejected up front
    big = M.Config.defaults(nx=1024, ny=1024, nz=1, pbc_x=-1, pbc_y=-1, pbc_z=0, precision=64)
    with M.Lattice(big) as lat:
        assert lat.demag_scratch_bytes() > 16 * 1024 * 1024
        m = torch.zeros((3, 1024 * 1024), dtype=torch.float64, device=dev)
        h = torch.zeros_like(m)
        with pytest.raises(M.MmcError, match="static array"):
            lat.demag_apply_static(m.data_ptr(), h.data_ptr(), None)
    # the sizes the header names: a 512 x 512 open film fits in FP32 (transform
    # grid 1023 x 1023), not in FP64; a 256 x 256 open film fits in FP64
    for side, prec, fits in ((512, 32, True), (512, 64, False), (256, 64, True)):
        c = M.Config.defaults(nx=side, ny=side, nz=1, pbc_x=0, pbc_y=0, pbc_z=0, precision=prec)
        with M.Lattice(c) as lat:
            assert (lat.demag_scratch_bytes() <= 16 * 1024 * 1024) == fits, (side, prec)
    # an unbuilt tensor is reported, not built (building allocates)
    small = M.Config.defaults(nx=16, ny=16, nz=1, precision=32)
    with M.Lattice(small) as lat:
        m = torch.zeros((3, 256), dtype=torch.float32, device=dev)
        h = torch.zeros_like(m)
        with pytest.raises(M.MmcError, match="not built"):
            lat.demag_apply_static(m.data_ptr(), h.data_ptr(), None)
    torch.cuda.synchronize()
