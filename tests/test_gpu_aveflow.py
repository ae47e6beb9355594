"""aveflow (aveflow.f95:5-200) on the device: the time averages, bit for bit the
oracle's, over a run of states and at the final step; and through whole steps against
the FP64 oracle.
"""
import numpy as np
import pytest

import lesgpu
from helpers import load_state, make_gpu, make_ref, random_state, rel_err, scenario

pytestmark = pytest.mark.gpu


def _same(gpu, orc, fid, what):
    g = gpu.download(fid)
    o = orc.get(fid).astype(np.float32)
    assert g.shape == o.shape, (what, g.shape, o.shape)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), (what, lesgpu.FIELD_NAMES[fid],
                                                                 float(np.abs(g - o).max()))


@pytest.mark.parametrize("shape,n1,nmax", [((40, 24, 12), 1, 4), ((37, 18, 11), 3, 6), ((64, 32, 9), 2, 2)])
def test_aveflow_matches_oracle_bitwise(built_lib, shape, n1, nmax):
    """A new random state (halos included) before every call: the accumulation, the
    zeroing at n1 (after garbage from earlier calls) and the finalisation at nmax."""
    sc = scenario(*shape, seed=201)
    gpu = make_gpu(sc, lesgpu.Params())
    orc = make_ref(4, sc, lesgpu.Params(), sqrt_half=1, red64=1)
    for n in range(1, nmax + 1):
        load_state(gpu, orc, random_state(sc, seed=300 + n))
        gpu.aveflow(n, n1, nmax)
        orc.aveflow(n, n1, nmax)
        if n < nmax and n >= n1:  # mid-run sums
            for fid in (lesgpu.AVEU, lesgpu.AVEW, lesgpu.UWFX, lesgpu.AVESMSM):
                _same(gpu, orc, fid, f"n={n}")
    for fid in lesgpu.AVE_FIELDS:
        _same(gpu, orc, fid, f"final n={nmax}")


def test_aveflow_over_steps_vs_fp64(built_lib):
    """The means against the FP64 oracle after whole steps.  The rms fields are left
    to the bitwise test: sqrt(|<u^2> - <u>^2|) in FP32 (the reference's formula)
    cancels catastrophically, so FP32 and FP64 runs differ there by far more than the
    inputs do."""
    sc = scenario(48, 32, 16, seed=202)
    params = lesgpu.Params(nmaxp=20)
    gpu = make_gpu(sc, params)
    orc = make_ref(8, sc, params, sqrt_half=0, red64=1)
    nmax = 5
    for n in range(1, nmax + 1):
        gpu.step(n, nmax)
        orc.step(n, nmax)
        gpu.aveflow(n, 2, nmax)
        orc.aveflow(n, 2, nmax)
    for fid in (lesgpu.AVEU, lesgpu.AVEV, lesgpu.AVEW, lesgpu.AVEP, lesgpu.AVESM):
        e = rel_err(gpu.download(fid).astype(np.float64), orc.get(fid))
        assert e <= 1e-4, (lesgpu.FIELD_NAMES[fid], e)


def test_aveflow_fields_need_a_first_call(built_lib):
    sc = scenario(24, 16, 8, seed=203)
    d = make_gpu(sc, lesgpu.Params())
    with pytest.raises(lesgpu.LesError):
        d.download(lesgpu.AVEU)
    with pytest.raises(lesgpu.LesError):
        d.aveflow(1, 3, 2)  # nmax < n1
    d.aveflow(1, 1, 1)
    assert d.download(lesgpu.AVEW).shape == (sc.im + 1, sc.jm, sc.km + 3)


def test_data10_data11_hold_the_averages(built_lib, tmp_path):
    """aveflow.f95:209-344: the files written at nmax, record by record, and byte for
    byte what the independent numpy writer makes of the downloaded averages."""
    import ftnio
    sc = scenario(33, 20, 10, seed=204)
    shape = (sc.im, sc.jm, sc.km)
    gpu = make_gpu(sc, lesgpu.Params(nmaxp=10))
    nmax = 4
    for n in range(1, nmax + 1):
        gpu.step(n, nmax)
        gpu.aveflow(n, 2, nmax)
    ids = {"aveu": lesgpu.AVEU, "avew": lesgpu.AVEW, "avev": lesgpu.AVEV, "aveuu": lesgpu.AVEUU,
           "aveww": lesgpu.AVEWW, "avevv": lesgpu.AVEVV, "uwfx": lesgpu.UWFX}
    for name, write, names in (("data10", gpu.write_data10, ftnio.DATA10), ("data11", gpu.write_data11, ftnio.DATA11)):
        p = str(tmp_path / name)
        write(p)
        want = {nm: gpu.download(ids[nm], (1, 1, 1), shape) for nm in names}
        got, _, _ = ftnio.read_fields(p, names, shape)
        for nm in names:
            assert np.array_equal(got[nm].view(np.uint32), want[nm].view(np.uint32)), (name, nm)
        q = p + ".np"
        ftnio.write_fields(q, want, names)
        assert open(p, "rb").read() == open(q, "rb").read(), name
    fresh = make_gpu(sc, lesgpu.Params())
    with pytest.raises(lesgpu.LesError, match="aveflow"):
        fresh.write_data10(str(tmp_path / "none"))
