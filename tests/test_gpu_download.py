"""Asynchronous downloads (les_gpu_download_async / _wait) through the C ABI.

A download is a snapshot in stream order: steps queued right after it must not change
what arrives, and every copy must equal what a synchronous download at the same point
of the time loop returns, bit for bit -- also when more copies are queued than the
handle has staging slots (8) and when boxes include halos.
"""
import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, scenario

pytestmark = pytest.mark.gpu


def _same(a, b, what):
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), what


def test_async_download_is_a_stream_ordered_snapshot(built_lib):
    sc = scenario(48, 30, 14, seed=101)
    params = lesgpu.Params(nmaxp=6)
    ref = make_gpu(sc, params)
    d = make_gpu(sc, params)
    fids = (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P)
    boxes = [None, ((1, 1, 1), (sc.im, sc.jm, sc.km)), ((0, 0, 0), (sc.im + 1, sc.jm + 1, sc.km + 1))]
    pending = []  # (ticket, array, step, fid, box)
    expect = {}
    nsteps = 5
    for n in range(1, nsteps + 1):
        ref.step(n, nsteps)
        for fid in fids:
            for q, box in enumerate(boxes):
                lb, ub = box if box else (None, None)
                expect[(n, fid, q)] = ref.download(fid, lb, ub)
        d.step(n, nsteps)  # queued; the downloads below snapshot its result
        for fid in fids:
            for q, box in enumerate(boxes):
                lb, ub = box if box else (None, None)
                out = np.zeros(expect[(n, fid, q)].shape, np.float32, order="F")
                pending.append((d.download_async(fid, out, lb, ub), out, n, fid, q))
    # 60 copies against 8 slots: the ring wrapped many times; wait in reverse order too
    for t, out, n, fid, q in reversed(pending):
        d.download_wait(t)
        _same(out, expect[(n, fid, q)], (n, lesgpu.FIELD_NAMES[fid], q))


def test_async_download_overlaps_following_steps(built_lib):
    """Queue a snapshot, then more steps before waiting: the copy holds the state at
    the snapshot, not the later one."""
    sc = scenario(40, 24, 12, seed=102)
    params = lesgpu.Params(nmaxp=4)
    d = make_gpu(sc, params)
    d.step(1, 4)
    snap = d.download(lesgpu.U)  # synchronous reference for the same point
    out = np.zeros(snap.shape, np.float32, order="F")
    t = d.download_async(lesgpu.U, out)
    for n in range(2, 5):
        d.step(n, 4)
    d.download_wait(t)
    _same(out, snap, "u after step 1")
    later = d.download(lesgpu.U)
    assert not np.array_equal(later, snap)  # the later steps did change u


def test_async_download_rejects_bad_input(built_lib):
    sc = scenario(24, 16, 8, seed=103)
    d = make_gpu(sc, lesgpu.Params())
    with pytest.raises(lesgpu.LesError):
        d.download_wait(12345)  # never issued
    with pytest.raises(lesgpu.LesError):
        d._check(d.lib.les_gpu_download_async(d._h, lesgpu.DX1, lesgpu._fptr(np.zeros(30, np.float32)),
                                              lesgpu._iarr((-1, 0, 0)), lesgpu._iarr((20, 0, 0)),
                                              lesgpu.C.byref(lesgpu.C.c_longlong())), "download_async")


@pytest.mark.parametrize("shape", [(48, 30, 14), (37, 9, 5)])
def test_download_boxes_equal_the_uploaded_array(built_lib, shape):
    """Every box shape: rows starting on a 16-byte word of the padded row with a width
    that is a multiple of 4 (the float4 pack) and all the others (the scalar pack)."""
    sc = scenario(*shape, seed=105)
    d = make_gpu(sc, lesgpu.Params())
    rng = np.random.default_rng(9)
    for fid in (lesgpu.U, lesgpu.P, lesgpu.SM):
        lb, ub = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
        full = np.asfortranarray(rng.standard_normal(tuple(ub[q] - lb[q] + 1 for q in range(3))).astype(np.float32))
        d.upload(fid, full)
        for i0, i1 in ((1, 4), (1, 8), (1, sc.im), (1, sc.im - 1), (2, 9), (max(lb[0], -3), ub[0]), (5, 12)):
            i0, i1 = max(i0, lb[0]), min(i1, ub[0])
            if i1 < i0:
                continue
            for (j0, j1), (k0, k1) in ((((lb[1], ub[1])), (lb[2], ub[2])), ((2, 3), (1, 2))):
                got = d.download(fid, (i0, j0, k0), (i1, j1, k1))
                want = full[i0 - lb[0]:i1 - lb[0] + 1, j0 - lb[1]:j1 - lb[1] + 1, k0 - lb[2]:k1 - lb[2] + 1]
                assert np.array_equal(got, want), (fid, (i0, j0, k0), (i1, j1, k1))
