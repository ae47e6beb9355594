"""Device-side set-up: the masks feedbfm (feedbfm.f95:87-116) makes on the device from
the heightmap, against the oracle's and the host's, and a domain set up from the host's
uploaded arrays stepping bit for bit like one set up on the device."""
import ctypes as C

import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, make_ref, scenario

pytestmark = pytest.mark.gpu

MASKS = (lesgpu.BMASK1, lesgpu.CMASK1, lesgpu.DMASK1)


def _host_setup(sc):
    """The host set-up arrays of les_gpu_setup_scenario, masks made on the host."""
    im, jm, km = sc.im, sc.jm, sc.km
    g = lesgpu.setup_grid(im, jm, km, sc.dx, sc.dy, sc.dz_law, sc.dz0, sc.dz_ratio)
    lib = lesgpu.load_library()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    cn = {n: np.zeros(s, np.float32) for n, s in (("cn2s", im), ("cn2l", im), ("cn3s", jm), ("cn3l", jm),
                                                  ("cn4s", km), ("cn4l", km))}
    assert lib.les_setup_poisson(im, jm, km, fp(g["dxs"]), fp(g["dys"]), fp(g["dzs"]), fp(cn["cn2s"]),
                                 fp(cn["cn2l"]), fp(cn["cn3s"]), fp(cn["cn3l"]), fp(cn["cn4s"]), fp(cn["cn4l"]),
                                 None) == 0
    zbm, uin, vin, win = lesgpu.generate_scenario(sc)
    masks = {lesgpu.BMASK1: np.zeros((im + 3, jm + 2, km + 2), np.float32, order="F"),
             lesgpu.CMASK1: np.zeros((im + 2, jm + 3, km + 2), np.float32, order="F"),
             lesgpu.DMASK1: np.zeros((im + 2, jm + 2, km + 2), np.float32, order="F")}
    assert lib.les_setup_masks(im, jm, km, fp(np.asfortranarray(zbm)), fp(g["z2"]), fp(g["dzn"]), None,
                               fp(masks[lesgpu.BMASK1]), fp(masks[lesgpu.CMASK1]), fp(masks[lesgpu.DMASK1])) == 0
    ones = {lesgpu.DX1: g["dx1"], lesgpu.DY1: g["dy1"], lesgpu.DZN: g["dzn"], lesgpu.DZS: g["dzs"],
            lesgpu.DXS: g["dxs"], lesgpu.DYS: g["dys"], lesgpu.Z2: g["z2"], lesgpu.CN2L: cn["cn2l"],
            lesgpu.CN2S: cn["cn2s"], lesgpu.CN3L: cn["cn3l"], lesgpu.CN3S: cn["cn3s"], lesgpu.CN4L: cn["cn4l"],
            lesgpu.CN4S: cn["cn4s"], lesgpu.UIN: uin, lesgpu.VIN: vin, lesgpu.WIN: win}
    return ones, masks, zbm


def test_device_masks_equal_the_oracles(built_lib):
    sc = scenario(37, 22, 13, seed=71, coverage=0.45)
    gpu = make_gpu(sc)
    orc = make_ref(4, sc)
    _, host, _ = _host_setup(sc)
    for fid in MASKS:
        g = gpu.download(fid)
        assert np.array_equal(g, orc.get(fid).astype(np.float32)), fid
        assert np.array_equal(g, host[fid]), fid
    d = gpu.download(lesgpu.DMASK1)
    assert 0.0 < d[1:-1, 1:-1, 1:-1].mean() < 1.0


@pytest.mark.parametrize("shape", [(48, 30, 14), (61, 9, 7)])
def test_uploaded_and_device_setup_step_alike(built_lib, shape):
    sc = scenario(*shape, seed=72, coverage=0.35)
    params = lesgpu.Params(nmaxp=12)
    a = make_gpu(sc, params)
    b = lesgpu.Domain(sc.im, sc.jm, sc.km, params)
    ones, masks, _ = _host_setup(sc)
    for fid, arr in ones.items():
        b.upload(fid, arr)
    for fid, arr in masks.items():
        b.upload(fid, arr)
    b.commit()
    for fid in MASKS:
        assert np.array_equal(a.download(fid), b.download(fid)), fid
    for n in range(1, 4):
        a.step(n, 3)
        b.step(n, 3)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), lesgpu.FIELD_NAMES[fid]
    assert a.diag() == b.diag()


def test_mask_upload_after_feedbfm_changes_that_mask_only(built_lib):
    sc = scenario(30, 16, 10, seed=73, coverage=0.5)
    gpu = make_gpu(sc)
    before = {fid: gpu.download(fid) for fid in MASKS}
    lb, ub = lesgpu.declared_extents(lesgpu.CMASK1, sc.im, sc.jm, sc.km)
    zero = np.zeros(tuple(ub[q] - lb[q] + 1 for q in range(3)), np.float32, order="F")
    gpu.upload(lesgpu.CMASK1, zero)
    gpu.commit()
    assert not gpu.download(lesgpu.CMASK1).any()
    for fid in (lesgpu.BMASK1, lesgpu.DMASK1):
        assert np.array_equal(gpu.download(fid), before[fid]), fid
    # and back through the device path
    _, _, zbm = _host_setup(sc)
    gpu.feedbfm(zbm)
    for fid in MASKS:
        assert np.array_equal(gpu.download(fid), before[fid]), fid


def test_feedbfm_needs_the_vertical_grid(built_lib):
    d = lesgpu.Domain(20, 10, 6, lesgpu.Params())
    with pytest.raises(lesgpu.LesError, match="z2 and dzn"):
        d.feedbfm(np.zeros((20, 10), np.float32))
