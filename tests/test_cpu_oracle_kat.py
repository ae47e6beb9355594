"""Known-answer checks of the CPU oracle, derived from the equations (no GPU).

The reference ships no golden vectors for the solver, so the oracle's restatement is
held to it by its loop-by-loop citations and by answers the equations fix exactly:
a uniform pressure with no forcing leaves velnw's velocities unchanged, a uniform
flow gives velfg no advection and only the wall function's diffusion at the first
level, adam maps a constant history to itself, feedbf does nothing where the building
masks are zero, press's SOR converges to a manufactured pressure, press removes the
volume-weighted mean of p, the oracle is deterministic, and FP32 drifts from FP64
within the 1e-4 budget of the parity contract.
"""
import numpy as np
import pytest

import lesgpu
from helpers import STATE, make_ref, manufactured_pressure, random_state, rel_err, scenario
from oracle import ref


@pytest.fixture(scope="module")
def oracle_built():
    ref.build()


def _loaded(prec, sc, params=None, seed=5, **kw):
    orc = make_ref(prec, sc, params or lesgpu.Params(), **kw)
    st = random_state(sc, seed=seed)
    for fid, a in st.items():
        orc.set(fid, a.astype(np.float64))
    return orc, st


def test_velnw_uniform_pressure_no_forcing_keeps_velocities(oracle_built):
    sc = scenario(20, 12, 8, seed=3)
    orc, st = _loaded(4, sc)
    lb, ub = orc.extents(lesgpu.P)
    orc.set(lesgpu.P, np.full(tuple(ub[q] - lb[q] + 1 for q in range(3)), 0.7))
    for fid in (lesgpu.F, lesgpu.G, lesgpu.H):
        orc.set(fid, np.zeros_like(st[fid], dtype=np.float64))
    orc.stage(ref.VELNW)
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W):
        assert np.array_equal(orc.get(fid).astype(np.float32), st[fid]), lesgpu.FIELD_NAMES[fid]


def uniform_flow(sc, U):
    """u = U, v = w = 0 over the full declared extents (halos too)."""
    out = {}
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W):
        lb, ub = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
        out[fid] = np.full(tuple(ub[q] - lb[q] + 1 for q in range(3)), U if fid == lesgpu.U else 0.0,
                           np.float32, order="F")
    return out


def velfg_uniform_expectation(f, g, h, km, U, vn, dzn1, tol):
    """velFG.f95:64-110 for u = U, v = w = 0: every advective flux cov1..9 and every
    gradient diu1..9 vanishes except the log-law wall gradient diu3(i,j,1) = U /
    (alog(0.5 dzn(1)/0.1) * 0.5 dzn(1)) of vel2.f95:138, so g = 0, h = 0 (k < km),
    f = 0 for k >= 2, and f(i,j,1) = vn * (-diu3(1) + 0) / dzn(1)."""
    # f, g, h over (0:im, 0:jm, 0:km): interior [1:, 1:, 1:]
    assert np.all(g[1:, 1:, 1:] == 0.0)
    assert np.all(h[1:, 1:, 1:km] == 0.0)
    assert np.all(f[1:, 1:, 2:] == 0.0)
    hz = 0.5 * dzn1
    f1 = -vn * (U / (np.log(hz / 0.1) * hz)) / dzn1
    got = f[1:, 1:, 1]
    assert np.all(np.abs(got - f1) <= tol * abs(f1)), (got.min(), got.max(), f1)


@pytest.mark.parametrize("prec", [4, 8])
def test_velfg_uniform_flow_has_no_advection(oracle_built, prec):
    sc = scenario(24, 14, 10, seed=3, coverage=0.0)
    params = lesgpu.Params()
    orc = make_ref(prec, sc, params)
    U = 3.0
    for fid, a in uniform_flow(sc, U).items():
        orc.set(fid, a.astype(np.float64))
    orc.stage(ref.VELFG)
    dzn1 = float(orc.get(lesgpu.DZN).ravel()[2])
    vn = float(np.float32(params.vn)) if prec == 4 else 15.83e-6
    velfg_uniform_expectation(orc.get(lesgpu.F), orc.get(lesgpu.G), orc.get(lesgpu.H), sc.km, U, vn, dzn1,
                              4e-7 if prec == 4 else 1e-13)


@pytest.mark.parametrize("prec,tol", [(8, 2e-7), (4, 3e-5)])
def test_press_sor_converges_to_a_manufactured_pressure(oracle_built, prec, tol):
    """press.f95:47-159 on rhs = A p* (A the SOR's own operator, press.f95:93-96):
    3000 fixed iterations from p = 0 reach p* minus its volume-weighted mean."""
    im, jm, km = 32, 16, 12
    sc = scenario(im, jm, km, seed=3, coverage=0.0)
    n = 3000
    o64 = make_ref(8, sc, lesgpu.Params(nmaxp=n, sor_fixed=1))
    u, expect = manufactured_pressure(o64, im, jm, km)
    orc = o64 if prec == 8 else make_ref(4, sc, lesgpu.Params(nmaxp=n, sor_fixed=1))
    for fid in (lesgpu.V, lesgpu.W, lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.P):
        lb, ub = orc.extents(fid)
        orc.set(fid, np.zeros(tuple(ub[q] - lb[q] + 1 for q in range(3))))
    orc.set(lesgpu.U, u.astype(np.float32).astype(np.float64) if prec == 4 else u)
    orc.stage(ref.PRESS, 2, 10)
    assert orc.diag()["iters"] == n
    p = orc.get(lesgpu.P, (1, 1, 1), (im, jm, km))
    assert rel_err(p, expect) <= tol, rel_err(p, expect)


def test_adam_keeps_a_constant_history(oracle_built):
    sc = scenario(20, 12, 8, seed=3)
    orc, st = _loaded(4, sc)
    for fid in (lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.FOLD, lesgpu.GOLD, lesgpu.HOLD):
        lb, ub = orc.extents(fid)
        orc.set(fid, np.full(tuple(ub[q] - lb[q] + 1 for q in range(3)), 2.0))
    orc.stage(ref.ADAM)
    for fid in (lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.FOLD, lesgpu.GOLD, lesgpu.HOLD):
        assert np.all(orc.get(fid, (1, 1, 1), (sc.im, sc.jm, sc.km)) == 2.0), lesgpu.FIELD_NAMES[fid]


def test_feedbf_does_nothing_without_buildings(oracle_built):
    sc = scenario(20, 12, 8, seed=3, coverage=0.0)
    orc, st = _loaded(4, sc)
    orc.stage(ref.FEEDBF)
    for fid in (lesgpu.F, lesgpu.G, lesgpu.H):
        assert np.array_equal(orc.get(fid).astype(np.float32), st[fid]), lesgpu.FIELD_NAMES[fid]
    for fid in (lesgpu.USUM, lesgpu.VSUM, lesgpu.WSUM):
        assert np.all(orc.get(fid, (1, 1, 1), (sc.im, sc.jm, sc.km)) == 0.0), lesgpu.FIELD_NAMES[fid]


@pytest.mark.parametrize("prec", [4, 8])
def test_press_removes_the_mean_pressure(oracle_built, prec):
    sc = scenario(20, 12, 8, seed=3)
    orc, _ = _loaded(prec, sc, lesgpu.Params(nmaxp=5))
    orc.stage(ref.PRESS, 2, 5)
    g = lesgpu.setup_grid(sc.im, sc.jm, sc.km)
    vol = (g["dx1"][2:2 + sc.im, None, None] * g["dy1"][1:1 + sc.jm][None, :, None]
           * g["dzn"][2:2 + sc.km][None, None, :]).astype(np.float64)
    p = orc.get(lesgpu.P, (1, 1, 1), (sc.im, sc.jm, sc.km))
    # the weights here are the FP32 grid; the FP64 oracle builds its own in double (1e-8 apart)
    assert abs((p * vol).sum()) <= (1e-6 if prec == 4 else 1e-7) * (np.abs(p) * vol).sum()


def test_oracle_is_deterministic(oracle_built):
    sc = scenario(20, 12, 8, seed=3)
    out = []
    for _ in range(2):
        orc = make_ref(4, sc, lesgpu.Params(nmaxp=10))
        for n in range(1, 4):
            orc.step(n, 3)
        out.append({fid: orc.get(fid) for fid in STATE})
    for fid in STATE:
        assert np.array_equal(out[0][fid], out[1][fid]), lesgpu.FIELD_NAMES[fid]


def test_fp32_stays_within_the_budget_of_fp64(oracle_built):
    """The parity contract's 1e-4 on u, v, w, p holds between the oracle's own FP32
    (the reference's real(kind=4)) and FP64 builds after 10 steps."""
    sc = scenario(24, 16, 20, seed=4)
    params = lesgpu.Params()
    a, b = make_ref(4, sc, params, sqrt_half=0, red64=0), make_ref(8, sc, params, sqrt_half=0, red64=1)
    for n in range(1, 11):
        a.step(n, 10)
        b.step(n, 10)
    lo, hi = (1, 1, 1), (sc.im, sc.jm, sc.km)
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P):
        assert rel_err(a.get(fid, lo, hi), b.get(fid, lo, hi)) <= 1e-4, lesgpu.FIELD_NAMES[fid]


def test_wall_at_rest_is_0_over_0(oracle_built):
    """vel2.f95:138,173 divide by the wall speeds uspd, vspd: at rest on the first level
    the reference forms 0/0.  The oracle's trap mode stops there and names the cell; by
    default it carries the NaN on, as the reference does (the GPU parity test checks the
    same NaN cells)."""
    sc = scenario(32, 16, 8, seed=57)
    st = random_state(sc, seed=157)
    for fid in (lesgpu.U, lesgpu.V):
        st[fid][8:15, 5:11, 1] = 0.0  # i 8..14, j 4..9 on k = 1
    orc = make_ref(4, sc, lesgpu.Params(nmaxp=3))
    for fid, a in st.items():
        orc.set(fid, a.astype(np.float64))
    orc.trap_wall(True)
    with pytest.raises(RuntimeError, match="0 by 0"):
        orc.stage(ref.VELFG)
    orc.trap_wall(False)
    for fid, a in st.items():
        orc.set(fid, a.astype(np.float64))
    orc.stage(ref.VELFG)
    f = orc.get(lesgpu.F)  # (0:im, 0:jm, 0:km)
    bad = np.argwhere(np.isnan(f[:, :, 1]))
    assert bad.size, "no NaN where the wall speed is zero"
    # every NaN of f at k = 1 lies next to the patch at rest (the faces of its cells)
    assert bad[:, 0].min() >= 7 and bad[:, 0].max() <= 15 and bad[:, 1].min() >= 4 and bad[:, 1].max() <= 10, bad
