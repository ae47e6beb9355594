"""The no-allocation entry point les_gpu_field_mean_noalloc, through the C ABI.

Some callers cannot allocate device memory at the moment they ask for a diagnostic:
code running under a device-memory cap sized before the run, a host framework whose
own allocator owns the device, or a monitor called between steps that must not put a
cudaMalloc/cudaFree on the step's timeline.  This entry point serves them: its scratch
is a static device array, so a call only launches kernels and copies.

Its value is press's pav reduction applied to any 3-D field: the volume-weighted
interior mean sum(x*dx1*dy1*dzn)/sum(dx1*dy1*dzn) (press.f95:124-133), rounded to
FP32.  It is checked against (a) an independent FP64 sum formed here with numpy and
(b) the existing entry point: with omega = 0 the SOR sweeps of press leave p
unchanged, so les_gpu_press then reports (les_gpu_diag, pav) the mean of the uploaded
p.  Two calls in a row check that the shared static scratch, left over from the first
call, does not leak into the second.  This file is collected last, so that a run that
stops at the first failure has run every other test before it.
"""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, random_state, scenario

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mpi-les_gb300", "csrc")


def _fn(dom: lesgpu.Domain):
    fn = dom.lib.les_gpu_field_mean_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    return fn


def _mean_noalloc(dom: lesgpu.Domain, fid: int) -> float:
    out = C.c_double(float("nan"))
    rc = _fn(dom)(dom._h, fid, C.byref(out))
    assert rc == 0, rc
    return out.value


def _ulps(a: float, b: float) -> int:
    x, y = np.float32(a), np.float32(b)
    return abs(int(x.view(np.int32)) - int(y.view(np.int32)))


def _fp64_mean(dom: lesgpu.Domain, x: np.ndarray, lb) -> float:
    """sum(x*dx1*dy1*dzn) / sum(dx1*dy1*dzn) over i=1..im, j=1..jm, k=1..km: each
    product rounded to FP32 left to right as press.f95:129-130 forms it, the sums
    exact (math.fsum), the quotient rounded to FP32 as press's pav is."""
    im, jm, km = dom.im, dom.jm, dom.km
    dx1 = dom.download(lesgpu.DX1).ravel()[2:2 + im]  # dx1(1..im) of (-1:im+1)
    dy1 = dom.download(lesgpu.DY1).ravel()[1:1 + jm]  # dy1(1..jm) of (0:jm+1)
    dzn = dom.download(lesgpu.DZN).ravel()[2:2 + km]  # dzn(1..km) of (-1:km+2)
    f32 = np.float32
    xi = x[1 - lb[0]:1 - lb[0] + im, 1 - lb[1]:1 - lb[1] + jm, 1 - lb[2]:1 - lb[2] + km].astype(f32)
    prod = ((xi * dx1.astype(f32)[:, None, None]).astype(f32) * dy1.astype(f32)[None, :, None]).astype(f32)
    prod = (prod * dzn.astype(f32)[None, None, :]).astype(f32)
    vol = ((dx1.astype(f32)[:, None, None] * dy1.astype(f32)[None, :, None]).astype(f32)
           * dzn.astype(f32)[None, None, :]).astype(f32)
    vol = np.broadcast_to(vol, prod.shape)
    return float(np.float32(math.fsum(prod.astype(np.float64).ravel()) / math.fsum(vol.astype(np.float64).ravel())))


def test_noalloc_source_calls_no_allocator():
    """The entry point's own code and the launcher it calls name no allocating routine."""
    src = open(os.path.join(CSRC, "les_noalloc.cu")).read()
    code = re.sub(r"//[^\n]*", "", src)
    for name in ("cudaMalloc", "cudaFree", "cudaMallocAsync", "cudaFreeAsync", "cudaMallocManaged",
                 "cudaMallocHost", "cudaHostAlloc", "cuMemAlloc", "malloc(", "new "):
        assert name not in code, name
    assert "static __device__ __align__(256)" in code
    assert "cudaGetSymbolAddress" in code
    kern = open(os.path.join(CSRC, "les_kernels.cu")).read()
    body = kern[kern.index("void les_launch_interior_mean("):]
    body = body[:body.index("\n}\n")]
    assert "Malloc" not in body and "Free" not in body


@pytest.mark.gpu
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
        assert _ulps(m, _fp64_mean(a, p, (0, 0, 0))) <= 1, (call, m)
        # the field itself is left as it was
        back = a.download(lesgpu.P)
        assert np.array_equal(back.view(np.uint32), p.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("fid", [lesgpu.U, lesgpu.SM, lesgpu.P])
def test_field_mean_noalloc_matches_fp64_sum(built_lib, fid):
    """Fields other than p, on a stretched vertical grid (dzn varies with k), two calls
    in a row, each within 1 FP32 ulp of the independent FP64 value."""
    sc = scenario(52, 26, 19, seed=73)
    d = make_gpu(sc)
    lb, _ = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
    for seed in (181, 182):
        x = random_state(sc, seed=seed)[fid]
        d.upload(fid, x)
        m = _mean_noalloc(d, fid)
        ref = _fp64_mean(d, x, lb)
        assert _ulps(m, ref) <= 1, (fid, seed, m, ref)


@pytest.mark.gpu
def test_field_mean_noalloc_allocates_nothing(built_lib):
    """After a first call (which looks up the static array's address and loads the
    kernels), later calls leave the device's free memory exactly as it was."""
    torch = pytest.importorskip("torch")
    sc = scenario(64, 40, 24, seed=75)
    d = make_gpu(sc)
    d.upload(lesgpu.P, random_state(sc, seed=191)[lesgpu.P])
    _mean_noalloc(d, lesgpu.P)
    d.sync()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        _mean_noalloc(d, lesgpu.P)
    d.sync()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


@pytest.mark.gpu
def test_field_mean_noalloc_rejects_large_domain(built_lib):
    """More reduction blocks than the static scratch holds: refused before any work
    (the check needs no set-up, so the domain is only created)."""
    im, jm, km = 3, 8192, 528  # 1 * 2048 * 33 = 67584 blocks > 65536
    assert ((im + 63) // 64) * ((jm + 3) // 4) * ((km + 15) // 16) > 65536
    d = lesgpu.Domain(im, jm, km, lesgpu.Params())
    out = C.c_double(0.0)
    assert _fn(d)(d._h, lesgpu.P, C.byref(out)) == -1  # LES_ERR_ARG
    buf = C.create_string_buffer(512)
    d.lib.les_gpu_last_error(d._h, buf, 512)
    assert b"static scratch" in buf.value, buf.value
    assert _fn(d)(d._h, 99, C.byref(out)) == -1  # not a 3-D field
    d.close()
