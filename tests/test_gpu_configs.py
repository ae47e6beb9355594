"""Parity at the configurations the throughput numbers are quoted on, against the FP64
oracle (the reference built with -freal-4-real-8), through the C ABI: max |x - x64| /
max |x64| over the interior of u, v, w and p within the contract's 1e-4.

  - the plain large domain, 600 x 600 x 90, 5 steps of 50 SOR iterations (the
    benchmark's own domain and seed);
  - three ensemble members of the uniform batch, 150 x 150 x 90 each with its own
    building seed, inflow direction in [0, 360) and speed in [2, 10] m/s, 20 steps,
    stepped together through les_batch_step;
  - uneven-batch shapes with kp = 48 and 64, with the power-law inflow and with the
    reference's 5 m/s inflow (bondv1.f95:33-54, whose k = 1..78 loop is cut to km here).
"""
import os

import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, make_ref, rel_err, scenario
from oracle import ref

pytestmark = pytest.mark.gpu
FIELDS = (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P)


def _fp64(sc, params, nsteps):
    ref.set_threads(os.cpu_count() or 1)
    orc = make_ref(8, sc, params, sqrt_half=0, red64=1, fast=True)
    for n in range(1, nsteps + 1):
        orc.step(n, nsteps)
    return orc


def _errors(dom, orc, sc):
    lo, hi = (1, 1, 1), (sc.im, sc.jm, sc.km)
    return {lesgpu.FIELD_NAMES[fid]: rel_err(dom.download(fid, lo, hi), orc.get(fid, lo, hi)) for fid in FIELDS}


@pytest.mark.slow
def test_bench_domain_600x600x90_vs_fp64(built_lib):
    sc = scenario(600, 600, 90, seed=1)  # bench.py's domain and seed
    params = lesgpu.Params()
    d = make_gpu(sc, params)
    for n in range(1, 6):
        d.step(n, 5)
    d.sync()
    assert d.nonfinite() == 0
    orc = _fp64(sc, params, 5)
    errs = _errors(d, orc, sc)
    orc.close()
    assert max(errs.values()) <= 1e-4, errs


@pytest.mark.parametrize("persistent", [False, True])
def test_uniform_batch_members_150x150x90_vs_fp64(built_lib, persistent):
    import random
    rng = random.Random(2024)
    scs = [scenario(150, 150, 90, seed=rng.getrandbits(48), direction_deg=rng.uniform(0.0, 360.0),
                    u_ref=rng.uniform(2.0, 10.0)) for _ in range(3)]
    params = lesgpu.Params()
    b = lesgpu.Batch(persistent_sor=persistent)
    doms = [make_gpu(sc, params) for sc in scs]
    for d in doms:
        b.add(d, 1, 20)
    while b.step() > 0:
        pass
    b.sync()
    for sc, d in zip(scs, doms):
        orc = _fp64(sc, params, 20)
        errs = _errors(d, orc, sc)
        orc.close()
        assert max(errs.values()) <= 1e-4, (sc.seed, sc.direction_deg, errs)
    b.close()


@pytest.mark.parametrize("shape", [(64, 256, 48), (192, 96, 64)])
@pytest.mark.parametrize("inflow_law", [1, 0])
def test_uneven_shapes_kp48_kp64_vs_fp64(built_lib, shape, inflow_law):
    # the reference's inflow is 5 m/s along x: no turn, so u(1,j,k) must read 5 m/s
    sc = scenario(*shape, seed=3000 + shape[2], coverage=0.3, direction_deg=250.0 if inflow_law else 0.0,
                  u_ref=6.0, inflow_law=inflow_law)
    params = lesgpu.Params()
    d = make_gpu(sc, params)
    for n in range(1, 11):
        d.step(n, 10)
    d.sync()
    orc = _fp64(sc, params, 10)
    errs = _errors(d, orc, sc)
    orc.close()
    assert max(errs.values()) <= 1e-4, errs
    if inflow_law == 0:  # the reference's inflow: 5 m/s on every level of the short column
        u = d.download(lesgpu.U, (1, 1, 1), (1, sc.jm, sc.km))
        assert np.allclose(u, 5.0, atol=2e-3)
