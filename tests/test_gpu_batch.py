"""Batches of resident domains (les_batch_*) and the serving loop on the GPU.

The contract of batching: a domain's result does not depend on the company it is
stepped in -- alone, in a batch, joined mid-way by others -- bit for bit.
"""
import numpy as np
import pytest

import lesgpu
import serve
from helpers import make_gpu, make_ref, rel_err, scenario

pytestmark = pytest.mark.gpu


def _alone(sc, params, nsteps):
    d = make_gpu(sc, params)
    for n in range(1, nsteps + 1):
        d.step(n, nsteps)
    d.sync()
    return d


def _same(a, b, what):
    for fid in lesgpu.STATE_FIELDS:
        x, y = a.download(fid), b.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (what, lesgpu.FIELD_NAMES[fid])


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_member_same_alone_and_in_mix(built_lib, persistent):
    params = lesgpu.Params(nmaxp=8)
    sa = scenario(48, 30, 14, seed=81, direction_deg=30.0, u_ref=4.0)
    sb = scenario(64, 40, 12, seed=82, direction_deg=200.0, u_ref=8.0)
    sc_ = scenario(37, 18, 11, seed=83, direction_deg=95.0)  # odd jm: the per-subroutine SOR path
    ref_a = _alone(sa, params, 6)
    ref_c = _alone(sc_, params, 4)
    b = lesgpu.Batch(persistent_sor=persistent)
    a, bb, c = make_gpu(sa, params), make_gpu(sb, params), make_gpu(sc_, params)
    sa_slot = b.add(a, 1, 6)
    b.add(bb, 1, 9)
    steps = 0
    while True:
        if steps == 2:
            sc_slot = b.add(c, 1, 4)  # joins mid-way
        live = b.step()
        steps += 1
        if live == 0 and steps > 2:
            break
    b.sync()
    assert b.progress(sa_slot) == (7, 6) and b.progress(sc_slot) == (5, 4)
    _same(a, ref_a, "a")
    _same(c, ref_c, "c")
    b.remove(sa_slot)
    b.close()


def test_batch_member_switches_to_narrow_sor_tiles(built_lib):
    """A 150-wide domain alone uses 32-column SOR tiles; as a batch member (the GPU
    shared) it moves to 16-column tiles, which waste fewer ring and padding columns,
    and marches k whole."""
    sc = scenario(150, 150, 8, seed=84)
    d = make_gpu(sc, lesgpu.Params(nmaxp=2))
    assert d.sor_shape()[0] == 32
    b = lesgpu.Batch()
    b.add(d, 1, 1)
    nx, ny, kchunk, depth = d.sor_shape()
    assert nx == 16 and kchunk == sc.km and depth == 1
    b.close()


def test_batch_members_vs_fp64_oracle(built_lib):
    """Ensemble members with their own seed, inflow direction and speed: each within
    the 1e-4 contract of the FP64 oracle after 8 steps."""
    params = lesgpu.Params()
    scs = [scenario(40, 24, 16, seed=91 + q, direction_deg=d, u_ref=s)
           for q, (d, s) in enumerate(((20.0, 3.0), (135.0, 9.0), (290.0, 6.0)))]
    b = lesgpu.Batch()
    doms = [make_gpu(sc, params) for sc in scs]
    for d in doms:
        b.add(d, 1, 8)
    while b.step() > 0:
        pass
    b.sync()
    for sc, d in zip(scs, doms):
        orc = make_ref(8, sc, params, sqrt_half=0, red64=1)
        for n in range(1, 9):
            orc.step(n, 8)
        for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P):
            g = d.download(fid, (1, 1, 1), (sc.im, sc.jm, sc.km)).astype(np.float64)
            o = orc.get(fid, (1, 1, 1), (sc.im, sc.jm, sc.km))
            assert rel_err(g, o) <= 1e-4, (sc.seed, lesgpu.FIELD_NAMES[fid])
    b.close()


def test_serving_small_stream_matches_alone(built_lib):
    """A short request stream through the server: every request completes, and a
    request's final state equals the same scenario stepped alone."""
    reqs = [serve.Request(q, 0.03 * q, im, jm, km, 100 + q, 37.0 * q, 3.0 + q, 0.3, steps)
            for q, (im, jm, km, steps) in enumerate(((32, 24, 10, 5), (48, 32, 12, 7), (40, 20, 9, 3),
                                                     (32, 32, 16, 6), (24, 16, 8, 4)))]
    be = serve.GpuBackend(reserve_bytes=1 << 30)
    kept = {}

    def on_done(r, dom):
        kept[r.rid] = {fid: dom.download(fid) for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P)}

    stats = serve.Server(be, setup_workers=2, on_done=on_done).run(reqs)
    assert stats["completed"] == len(reqs) and stats["rejected"] == 0
    assert stats["latency_s"]["p99"] is not None
    for r in (reqs[1], reqs[3]):
        alone = _alone(be.scenario(r), lesgpu.Params(), r.steps)
        for fid, x in kept[r.rid].items():
            y = alone.download(fid)
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (r.rid, lesgpu.FIELD_NAMES[fid])
    be.batch.close()


def test_batched_sor_groups_and_fallbacks_match_alone(built_lib):
    """Members of two tile shapes (two batched SOR launches), a member whose SOR cannot
    be batched (odd jm: the per-subroutine sweep) and a member at its first step, all in
    one batch: each ends bitwise equal to the same domain stepped alone, and a batched
    member issues fewer launches of its own than its whole-step graph would."""
    params = lesgpu.Params(nmaxp=12)
    specs = [(scenario(150, 60, 14, seed=301, direction_deg=10.0), (32, 24, 0, 1)),
             (scenario(120, 48, 12, seed=302, direction_deg=140.0), (16, 20, 0, 1)),
             (scenario(96, 40, 10, seed=303, direction_deg=250.0), (32, 20, 0, 1)),
             (scenario(40, 21, 9, seed=304), None)]
    alone = []
    for sc, shape in specs:
        d = make_gpu(sc, params)
        if shape:
            d.set_sor_shape(*shape)
        for n in range(1, 6):
            d.step(n, 5)
        d.sync()
        alone.append(d)
    b = lesgpu.Batch(persistent_sor=True)
    doms = []
    for sc, shape in specs:
        d = make_gpu(sc, params)
        if shape:
            d.set_sor_shape(*shape)
        doms.append(d)
        b.add(d, 1, 5)
    l0 = doms[0].launch_count()
    while b.step() > 0:
        pass
    b.sync()
    per_step = (doms[0].launch_count() - l0) / 5
    for q, (x, y) in enumerate(zip(doms, alone)):
        _same(x, y, f"member {q}")
    whole = make_gpu(specs[0][0], params)
    whole.set_sor_shape(*specs[0][1])
    whole.step(1, 5)
    w0 = whole.launch_count()
    whole.step(2, 5)
    assert per_step < (whole.launch_count() - w0) - params.nmaxp + 5, per_step
    b.close()


def test_batched_sor_wait_gives_up_and_reports(built_lib):
    """A dependency wait of the persistent SOR launch that can never end (a member held
    on a count nothing reaches) gives up after its bound, the launch stops, and
    les_batch_sync reports it; the GPU stays usable and the next batch steps normally."""
    params = lesgpu.Params(nmaxp=6)
    b = lesgpu.Batch(persistent_sor=True)
    doms = [make_gpu(scenario(64, 40, 12, seed=311 + q), params) for q in range(2)]
    slots = [b.add(d, 1, 3) for d in doms]
    b.set_wait_limit(1 << 14, hold_slot=slots[0])  # about 2 ms of polling
    b.step()
    with pytest.raises(RuntimeError, match="gave up"):
        b.sync()
    b.set_wait_limit(1 << 23, hold_slot=-1)
    b.close()
    # a fresh batch on the same GPU: steps and matches the domain alone
    sc = scenario(64, 40, 12, seed=321)
    ref = _alone(sc, params, 3)
    b2 = lesgpu.Batch(persistent_sor=True)
    d = make_gpu(sc, params)
    b2.add(d, 1, 3)
    while b2.step() > 0:
        pass
    b2.sync()
    _same(d, ref, "after a failed wait")
    b2.close()


def test_batched_sor_member_replaced_matches_alone(built_lib):
    """A finished member removed and destroyed, then a new domain of the same shape
    created (its handle and device buffers may take the freed addresses) and added to
    the same persistent-SOR batch: the batch rebuilds its member table for the new
    domain, which ends bitwise equal to the same scenario stepped alone."""
    params = lesgpu.Params(nmaxp=8)
    sa = scenario(64, 40, 12, seed=331, direction_deg=20.0)
    sb = scenario(64, 40, 12, seed=332, direction_deg=160.0, u_ref=7.0)
    keep = scenario(48, 32, 12, seed=333)
    ref_b = _alone(sb, params, 4)
    ref_k = _alone(keep, params, 7)
    b = lesgpu.Batch(persistent_sor=True)
    a = make_gpu(sa, params)
    k = make_gpu(keep, params)
    sa_slot = b.add(a, 1, 3)
    b.add(k, 1, 7)
    for _ in range(3):
        b.step()
    b.sync()
    b.remove(sa_slot).close()
    d = make_gpu(sb, params)
    b.add(d, 1, 4)
    while b.step() > 0:
        pass
    b.sync()
    _same(d, ref_b, "replacement")
    _same(k, ref_k, "kept member")
    b.close()
