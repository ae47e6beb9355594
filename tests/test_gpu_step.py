"""Whole-step parity: the GPU time loop against the FP32 and FP64 oracles.

The parity contract: after N steps, err(x) = max|x - x_ref| / max|x_ref| over the
interior is <= 1e-4 for u, v, w and p against the FP64 oracle.  Against the FP32
oracle the GPU is exact except for the order of the FP64 sums (rhsav, pav) and,
with the oracle in gfortran mode, glibc's powf(x, 0.5) for x**0.5; the tighter
tolerances below bound those.
"""
import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, make_ref, rel_err, scenario

pytestmark = pytest.mark.gpu

FIELDS = ((lesgpu.U, "u"), (lesgpu.V, "v"), (lesgpu.W, "w"), (lesgpu.P, "p"))


def _interior(obj, fid, sc, gpu):
    lb, ub = (1, 1, 1), (sc.im, sc.jm, sc.km)
    if gpu:
        return obj.download(fid, lb, ub).astype(np.float64)
    return obj.get(fid, lb, ub)


def _run_pair(sc, nsteps, params, prec, **rkw):
    gpu = make_gpu(sc, params)
    orc = make_ref(prec, sc, params, **rkw)
    for n in range(1, nsteps + 1):
        gpu.step(n, nsteps)
        orc.step(n, nsteps)
    gpu.sync()
    return gpu, orc


@pytest.mark.parametrize("shape,nmaxp", [((48, 32, 16), 20), ((130, 46, 12), 7), ((37, 6, 9), 9),
                                         ((61, 21, 10), 6), ((250, 100, 20), 50), ((121, 2, 5), 3),
                                         ((50, 30, 12), 1)])
def test_step_matches_stage_sequence(built_lib, shape, nmaxp):
    """The fused/graph step equals the per-subroutine entry points bit for bit.

    Shapes cover partial SOR tiles in i and j, jm smaller than a tile, an odd jm (the
    per-subroutine SOR path), jm = 2 and an odd iteration count (copy-back)."""
    sc = scenario(*shape, seed=9)
    params = lesgpu.Params(nmaxp=nmaxp)
    a = make_gpu(sc, params)
    b = make_gpu(sc, params)
    for n in range(1, 5):
        a.step(n, 4)
        b.velnw(); b.bondv1(n); b.velfg(); b.feedbf(); b.les(); b.adam(); b.press(n, 4)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), lesgpu.FIELD_NAMES[fid]
    da, db = a.diag(), b.diag()
    assert da["iters"] == db["iters"] == nmaxp
    assert abs(da["sor"] - db["sor"]) <= 1e-5 * abs(db["sor"])


def test_step_after_uploading_state(built_lib):
    """An uploaded p (halos not matching its interior) is handled exactly."""
    from helpers import random_state
    sc = scenario(64, 40, 12, seed=31)
    params = lesgpu.Params(nmaxp=10)
    a = make_gpu(sc, params)
    b = make_gpu(sc, params)
    st = random_state(sc, seed=77)
    for fid, arr in st.items():
        a.upload(fid, arr)
        b.upload(fid, arr)
    for n in range(2, 5):
        a.step(n, 9)
        b.velnw(); b.bondv1(n); b.velfg(); b.feedbf(); b.les(); b.adam(); b.press(n, 9)
        for fid in lesgpu.STATE_FIELDS:
            x, y = a.download(fid), b.download(fid)
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (n, lesgpu.FIELD_NAMES[fid])


@pytest.mark.parametrize("kchunk", [3, 5, 8])
def test_sor_k_chunks_match_one_chunk(built_lib, monkeypatch, kchunk):
    """The SOR march split into k chunks (each starting with a recomputed red plane)
    gives the single-chunk result bit for bit; only the residual's summation order
    differs."""
    sc = scenario(64, 24, 30, seed=71)
    params = lesgpu.Params(nmaxp=9)

    def run(chunk):
        monkeypatch.setenv("LES_SOR_KCHUNK", str(chunk))
        d = make_gpu(sc, params)
        for n in range(1, 5):
            d.step(n, 4)
        d.sync()
        return d

    a, b = run(1000), run(kchunk)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), lesgpu.FIELD_NAMES[fid]
    da, db = a.diag(), b.diag()
    assert da["iters"] == db["iters"] == 9
    assert abs(da["sor"] - db["sor"]) <= 1e-6 * abs(da["sor"])


@pytest.mark.parametrize("shape", [(16, 16, 0), (16, 20, 0), (16, 24, 0), (16, 28, 0), (32, 20, 0), (32, 28, 5),
                                   (16, 24, 5), (16, 28, 3), (32, 24, 0, 2), (32, 28, 0, 2), (32, 32, 0, 2)])
def test_sor_tile_shapes_match(built_lib, shape):
    """Every tile shape of the fused SOR sweep -- 16- and 32-column tiles, each tile
    height, k chunks of either, and two iterations per k-march -- gives the same fields
    bit for bit.  130 cells wide: three 16-column tiles (the last one partial) against
    two 32-column ones; 36 rows: partial tiles in j for every height."""
    sc = scenario(130, 36, 14, seed=73)
    params = lesgpu.Params(nmaxp=9)

    def run(nx, ny, kchunk, depth=1):
        d = make_gpu(sc, params)
        d.set_sor_shape(nx, ny, kchunk, depth)
        for n in range(1, 5):
            d.step(n, 4)
        d.sync()
        return d

    a, b = run(32, 24, 1000, 1), run(*shape)
    assert a.sor_shape() == (32, 24, 14, 1)
    nx, ny, kchunk = shape[:3]
    depth = shape[3] if len(shape) > 3 else 1
    assert b.sor_shape() == (nx, ny, kchunk if kchunk else 14, depth)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (shape, lesgpu.FIELD_NAMES[fid])
    da, db = a.diag(), b.diag()
    assert da["iters"] == db["iters"] == 9
    assert abs(da["sor"] - db["sor"]) <= 1e-6 * abs(da["sor"])


def test_sor_shape_rejects_unbuilt_shapes(built_lib):
    d = lesgpu.Domain(40, 20, 8, lesgpu.Params())
    for bad in ((8, 24, 0), (32, 32, 0), (32, 24, -1), (32, 32, 0, 1), (16, 24, 0, 2), (32, 20, 0, 2),
                (32, 24, 4, 2), (32, 24, 0, 3)):
        with pytest.raises(lesgpu.LesError):
            d.set_sor_shape(*bad)


@pytest.mark.parametrize("nmaxp", [2, 3, 8, 9, 50])
@pytest.mark.parametrize("shape", [(150, 60, 20), (64, 6, 12), (40, 4, 7), (64, 2, 12)])
def test_two_iteration_sor_matches_one_iteration(built_lib, nmaxp, shape):
    """Two SOR iterations per k-march give the fields of one iteration per launch bit
    for bit, for even and odd iteration counts (a one-iteration launch before or after
    the pairs), partial tiles, jm = 4 and 6 (ghost rows that are copies of copies), and
    the residual of the last iteration within summation-order rounding.  jm = 2 (too
    narrow for the four-row ghost band) runs one iteration per launch."""
    sc = scenario(*shape, seed=75)
    params = lesgpu.Params(nmaxp=nmaxp)

    def run(depth):
        d = make_gpu(sc, params)
        d.set_sor_shape(32, 24 if depth == 1 else 28, 0, depth)
        for n in range(1, 4):
            d.step(n, 3)
        d.sync()
        return d

    a, b = run(1), run(2)
    assert b.sor_shape()[3] == (2 if sc.jm >= 4 else 1)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (nmaxp, lesgpu.FIELD_NAMES[fid])
    da, db = a.diag(), b.diag()
    assert da["iters"] == db["iters"] == nmaxp
    assert abs(da["sor"] - db["sor"]) <= 1e-6 * abs(da["sor"])
    # the per-subroutine press on the same plan gives the same fields as the graph step
    c = make_gpu(sc, params)
    c.set_sor_shape(32, 28, 0, 2)
    for n in range(1, 4):
        c.velnw(); c.bondv1(n); c.velfg(); c.feedbf(); c.les(); c.adam(); c.press(n, 3)
    for fid in lesgpu.STATE_FIELDS:
        x, y = b.download(fid), c.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (nmaxp, lesgpu.FIELD_NAMES[fid])


@pytest.mark.parametrize("spacing", [(4.0, 4.0), (3.0, 5.0)])
def test_step_reciprocal_division_matches_ieee(built_lib, monkeypatch, spacing):
    """The reciprocal-corrected divisions (and the power-of-two multiplications) give
    the same step as IEEE divisions everywhere, bit for bit."""
    sc = scenario(48, 30, 14, seed=61, dx=spacing[0], dy=spacing[1])
    params = lesgpu.Params(nmaxp=8)
    a = make_gpu(sc, params)
    monkeypatch.setenv("LES_IEEE_DIV", "1")
    b = make_gpu(sc, params)
    monkeypatch.delenv("LES_IEEE_DIV")
    for n in range(1, 6):
        a.step(n, 5)
        b.step(n, 5)
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), lesgpu.FIELD_NAMES[fid]


@pytest.mark.parametrize("shape,nsteps,spacing", [((48, 32, 24), 10, (4.0, 4.0)), ((40, 64, 20), 6, (4.0, 4.0)),
                                                  ((44, 30, 16), 6, (3.0, 5.0))])
def test_steps_vs_fp32_oracle(built_lib, shape, nsteps, spacing):
    sc = scenario(*shape, seed=21, dx=spacing[0], dy=spacing[1])
    params = lesgpu.Params()
    gpu, orc = _run_pair(sc, nsteps, params, 4, sqrt_half=1, red64=1)
    for fid, nm in FIELDS:
        e = rel_err(_interior(gpu, fid, sc, True), _interior(orc, fid, sc, False))
        assert e <= 1e-5, (nm, e)
    assert gpu.diag()["iters"] == orc.diag()["iters"]


@pytest.mark.parametrize("shape,nsteps", [((48, 32, 24), 10)])
def test_steps_vs_fp64_oracle(built_lib, shape, nsteps):
    sc = scenario(*shape, seed=22)
    params = lesgpu.Params()
    gpu, orc = _run_pair(sc, nsteps, params, 8, sqrt_half=0, red64=1)
    for fid, nm in FIELDS:
        e = rel_err(_interior(gpu, fid, sc, True), _interior(orc, fid, sc, False))
        assert e <= 1e-4, (nm, e)


def test_steps_vs_gfortran_semantics(built_lib):
    """Oracle with powf(x,0.5) and sequential FP32 sums, exactly as the reference."""
    sc = scenario(48, 32, 24, seed=23)
    params = lesgpu.Params()
    gpu, orc = _run_pair(sc, 8, params, 4, sqrt_half=0, red64=0)
    for fid, nm in FIELDS:
        e = rel_err(_interior(gpu, fid, sc, True), _interior(orc, fid, sc, False))
        assert e <= 1e-4, (nm, e)


@pytest.mark.slow
def test_plain_small_config_vs_fp64(built_lib):
    """The plain small configuration: 150x150x90, 20 steps, 50 SOR iterations."""
    sc = scenario(150, 150, 90, seed=1)
    params = lesgpu.Params()
    gpu, orc = _run_pair(sc, 20, params, 8, sqrt_half=0, red64=1, fast=True)
    errs = {nm: rel_err(_interior(gpu, fid, sc, True), _interior(orc, fid, sc, False)) for fid, nm in FIELDS}
    assert max(errs.values()) <= 1e-4, errs
    assert gpu.nonfinite() == 0


def test_steps_vs_committed_golden(built_lib):
    """The solver against the committed oracle fixtures (tests/golden): within 1e-4 of
    the gfortran-semantics FP32 run and of the FP64 run (the parity contract)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_30x20x16_s8.npz"))
    sc = scenario(30, 20, 16, seed=8)
    gpu = make_gpu(sc, lesgpu.Params(nmaxp=50))
    for n in range(1, 4):
        gpu.step(n, 3)
    gpu.sync()
    for fid, nm in FIELDS:
        x = _interior(gpu, fid, sc, True)
        for prec in (32, 64):
            e = rel_err(x, g[f"{nm}{prec}"].astype(np.float64))
            assert e <= 1e-4, (nm, prec, e)
    assert gpu.diag()["iters"] == int(g["diag32"][0])


@pytest.mark.parametrize("depth", [1, 2])
@pytest.mark.parametrize("pjuge,lo,hi", [(12000.0, 2, 48), (40000.0, 1, 6)])
def test_sor_early_exit_like_the_reference(built_lib, pjuge, lo, hi, depth):
    """press.f95:119-121: the SOR loop exits once sor < pjuge.  With thresholds the
    residual crosses mid-loop (and after the first iteration), the whole-step graph
    and the per-subroutine calls stop at the oracle's iteration in every step -- also
    when two iterations share a k-march and the first of them met the test (the launch
    is cut back to it)."""
    sc = scenario(40, 24, 12, seed=5)
    params = lesgpu.Params(sor_fixed=0, pjuge=pjuge)
    gpu = make_gpu(sc, params)
    stages = make_gpu(sc, params)
    for d in (gpu, stages):
        d.set_sor_shape(32, 24 if depth == 1 else 28, 0, depth)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    iters = []
    for n in range(1, 6):
        gpu.step(n, 5)
        stages.velnw(); stages.bondv1(n); stages.velfg(); stages.feedbf(); stages.les(); stages.adam()
        stages.press(n, 5)
        orc.step(n, 5)
        want = orc.diag()["iters"]
        assert gpu.diag()["iters"] == want, (n, gpu.diag(), orc.diag())
        assert stages.diag()["iters"] == want, (n, stages.diag(), orc.diag())
        iters.append(want)
    assert lo <= min(iters) and max(iters) <= hi, iters
    for fid, nm in FIELDS:
        e = rel_err(_interior(gpu, fid, sc, True), _interior(orc, fid, sc, False))
        assert e <= 1e-5, (nm, e)
        x, y = gpu.download(fid), stages.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), nm


def test_profile_modes(built_lib):
    """les_gpu_profile: every stage times to a positive figure; the sweep-only SOR figure
    times the fused sweeps after the first; a single-iteration SOR has none to time."""
    sc = scenario(64, 40, 16, seed=71)
    d = make_gpu(sc, lesgpu.Params(nmaxp=12))
    d.step(1, 5)
    for what in (lesgpu.PROF_SOR, lesgpu.PROF_VELFG, lesgpu.PROF_LES, lesgpu.PROF_VELNW, lesgpu.PROF_STEP,
                 lesgpu.PROF_SOR_SWEEP):
        ms = d.profile(what, 3)
        assert 0.0 < ms < 1e3, (what, ms)
    assert d.nonfinite() == 0
    one = make_gpu(sc, lesgpu.Params(nmaxp=1))
    with pytest.raises(lesgpu.LesError, match="no fused sweeps"):
        one.profile(lesgpu.PROF_SOR_SWEEP, 2)


@pytest.mark.parametrize("omega", [1.0, 1.3])
def test_steps_with_relaxation_factor(built_lib, omega):
    """omega of press.f95:45 (1 in the reference; the TMA sweep is built for it, any
    other value runs the register sweep): the step graph equals the per-subroutine
    sequence bit for bit, and both follow the FP32 oracle."""
    sc = scenario(48, 32, 12, seed=73)
    params = lesgpu.Params(omega=omega, nmaxp=15)
    a = make_gpu(sc, params)
    b = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    for n in range(1, 4):
        a.step(n, 3)
        b.velnw(); b.bondv1(n); b.velfg(); b.feedbf(); b.les(); b.adam(); b.press(n, 3)
        orc.step(n, 3)
    for fid, nm in FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), nm
        e = rel_err(_interior(a, fid, sc, True), _interior(orc, fid, sc, False))
        assert e <= 1e-5, (nm, e)
