"""Equation-derived known answers on the GPU, through the C ABI (the same cases the
oracle is held to in test_cpu_oracle_kat.py): a uniform flow gives velfg no advection
(velFG.f95:64-110, vel2.f95:74-197) and press's SOR converges to a manufactured
pressure (press.f95:47-159)."""
import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, make_ref, manufactured_pressure, rel_err, scenario
from test_cpu_oracle_kat import uniform_flow, velfg_uniform_expectation

pytestmark = pytest.mark.gpu


def test_velfg_uniform_flow_has_no_advection_gpu(built_lib):
    sc = scenario(40, 18, 12, seed=3, coverage=0.0)
    d = make_gpu(sc)
    U = 3.0
    for fid, a in uniform_flow(sc, U).items():
        d.upload(fid, a)
    d.velfg()
    dzn1 = float(d.download(lesgpu.DZN).ravel()[2])
    velfg_uniform_expectation(d.download(lesgpu.F), d.download(lesgpu.G), d.download(lesgpu.H), sc.km, U,
                              float(np.float32(d.params.vn)), dzn1, 4e-7)


# (shape, iterations, tolerance): the FP32 fixed point's distance from p* grows with the
# operator's condition number (the oracle's FP32 build stops at 7e-6 and 1e-4 here)
@pytest.mark.parametrize("shape,n,tol", [((32, 16, 12), 3000, 3e-5), ((130, 24, 10), 20000, 2e-4)])
def test_press_sor_converges_to_a_manufactured_pressure_gpu(built_lib, shape, n, tol):
    im, jm, km = shape
    sc = scenario(im, jm, km, seed=3, coverage=0.0)
    o64 = make_ref(8, sc, lesgpu.Params(nmaxp=n, sor_fixed=1))
    u, expect = manufactured_pressure(o64, im, jm, km)
    d = make_gpu(sc, lesgpu.Params(nmaxp=n, sor_fixed=1))
    for fid in (lesgpu.V, lesgpu.W, lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.P):
        lb, ub = lesgpu.declared_extents(fid, im, jm, km)
        d.upload(fid, np.zeros(tuple(ub[q] - lb[q] + 1 for q in range(3)), np.float32, order="F"))
    d.upload(lesgpu.U, u.astype(np.float32))
    d.press(2, 10)
    assert d.diag()["iters"] == n
    p = d.download(lesgpu.P, (1, 1, 1), (im, jm, km))
    assert rel_err(p, expect) <= tol, rel_err(p, expect)
