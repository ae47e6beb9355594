"""The no-allocation entry point les_gpu_field_mean_noalloc, through the C ABI.

Its value is press's pav: the volume-weighted interior mean of p, rounded to FP32.
With omega = 0 the SOR sweeps of press leave p unchanged, so les_gpu_press then
reports (les_gpu_diag, pav) the mean of the p that was uploaded -- the existing entry
point's output that the new one must reproduce.  Two calls in a row check that the
shared static scratch, left over from the first call, does not leak into the second.
"""
import ctypes as C

import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, random_state, scenario

pytestmark = pytest.mark.gpu


def _mean_noalloc(dom: lesgpu.Domain, fid: int) -> float:
    fn = dom.lib.les_gpu_field_mean_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    out = C.c_double(float("nan"))
    rc = fn(dom._h, fid, C.byref(out))
    assert rc == 0, rc
    return out.value


def _ulps(a: float, b: float) -> int:
    x, y = np.float32(a), np.float32(b)
    return abs(int(x.view(np.int32)) - int(y.view(np.int32)))


@pytest.mark.parametrize("shape", [(48, 30, 14), (37, 18, 11)])
def test_field_mean_noalloc_matches_press_pav(built_lib, shape):
    sc = scenario(*shape, seed=71)
    params = lesgpu.Params(omega=0.0, nmaxp=2)
    a = make_gpu(sc, params)  # the new entry point
    b = make_gpu(sc, params)  # press, the existing one
    for call, seed in enumerate((171, 172)):
        p = random_state(sc, seed=seed)[lesgpu.P]
        p = np.asfortranarray(p + np.float32(0.25 * (call + 1)))  # a clearly nonzero mean
        a.upload(lesgpu.P, p)
        b.upload(lesgpu.P, p)
        m = _mean_noalloc(a, lesgpu.P)
        b.press(call + 1, 10)
        pav = b.diag()["pav"]
        assert _ulps(m, pav) <= 1, (call, m, pav)
        assert np.float32(m) == np.float32(m)  # finite, not the NaN it started as
        # the field itself is left as it was
        back = a.download(lesgpu.P)
        assert np.array_equal(back.view(np.uint32), p.view(np.uint32))


def test_field_mean_noalloc_rejects_large_domain(built_lib):
    """More interior blocks than the static scratch holds: refused before any work
    (the check needs no set-up, so the domain is only created)."""
    im, jm, km = 3, 4096, 260  # 1 * 1024 * 260 = 266240 blocks > 262144
    d = lesgpu.Domain(im, jm, km, lesgpu.Params())
    fn = d.lib.les_gpu_field_mean_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    out = C.c_double(0.0)
    assert fn(d._h, lesgpu.P, C.byref(out)) == -1  # LES_ERR_ARG
    buf = C.create_string_buffer(512)
    d.lib.les_gpu_last_error(d._h, buf, 512)
    assert b"static scratch" in buf.value, buf.value
    assert fn(d._h, 99, C.byref(out)) == -1  # not a 3-D field
