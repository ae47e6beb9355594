"""Known-answer checks of the CPU oracle, derived from the equations (no GPU).

The reference ships no golden vectors for the solver, so the oracle's restatement is
held to it by its loop-by-loop citations and by answers the equations fix exactly:
a uniform pressure with no forcing leaves velnw's velocities unchanged, adam maps a
constant history to itself, feedbf does nothing where the building masks are zero,
press removes the volume-weighted mean of p, the oracle is deterministic, and FP32
drifts from FP64 within the 1e-4 budget of the parity contract.
"""
import numpy as np
import pytest

import lesgpu
from helpers import STATE, make_ref, random_state, rel_err, scenario
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
