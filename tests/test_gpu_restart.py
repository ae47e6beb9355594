"""The reference's result and restart files from device state (press.f95:205-216,
adam.f95:20-27, anime.f95:326-595) and the restart read (ifdata.f95:252-480): the
library's bytes against the independent numpy writer, and a restarted run against a
continuous one and the oracle."""
import os

import numpy as np
import pytest

import ftnio
import lesgpu
from helpers import make_gpu, make_ref, rel_err, scenario

pytestmark = pytest.mark.gpu

IDS = {"u": lesgpu.U, "v": lesgpu.V, "w": lesgpu.W, "p": lesgpu.P, "usum": lesgpu.USUM, "vsum": lesgpu.VSUM,
       "wsum": lesgpu.WSUM, "f": lesgpu.F, "g": lesgpu.G, "h": lesgpu.H, "fold": lesgpu.FOLD,
       "gold": lesgpu.GOLD, "hold": lesgpu.HOLD}


def _interiors(gpu, names, shape):
    out = {}
    for nm in names:
        if nm == "fghold":  # never assigned in the reference: zeros
            out[nm] = np.zeros(shape, np.float32, order="F")
        else:
            out[nm] = gpu.download(IDS[nm], (1, 1, 1), shape)
    return out


def _same(a, b, what):
    assert a.shape == b.shape, what
    assert np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32)), what


def _stepped(sc, nsteps, params=None):
    gpu = make_gpu(sc, params or lesgpu.Params())
    for n in range(1, nsteps + 1):
        gpu.step(n, 20)
    return gpu


@pytest.mark.parametrize("big_endian", [True, False])
def test_files_hold_the_device_state(built_lib, tmp_path, big_endian):
    sc = scenario(40, 24, 12, seed=61)
    shape = (sc.im, sc.jm, sc.km)
    gpu = _stepped(sc, 3)
    t = np.float32(2) * np.float32(0.05)
    files = {
        "data20": (gpu.write_data20, ftnio.DATA20, None),
        "data21": (gpu.write_data21, ftnio.DATA21, None),
        "data30": (lambda p, big_endian: gpu.write_data30(p, 3, float(t), big_endian), ftnio.DATA30, (3, t)),
        "data31": (gpu.write_data31, ftnio.DATA31, None),
    }
    for name, (write, names, head) in files.items():
        p = str(tmp_path / name)
        write(p, big_endian=big_endian)
        want = _interiors(gpu, names, shape)
        got, n, tt = ftnio.read_fields(p, names, shape, header=head is not None)
        assert ftnio.detect_order(p) is big_endian
        for nm in names:
            _same(got[nm], want[nm], (name, nm))
        if head is not None:
            assert (n, np.float32(tt)) == head
        q = str(tmp_path / (name + ".np"))
        ftnio.write_fields(q, want, names, big_endian, header=head)
        assert open(p, "rb").read() == open(q, "rb").read(), name


def test_subrecords_and_little_endian_read_back(built_lib, tmp_path, monkeypatch):
    """A lowered subrecord limit (gfortran's -fmax-subrecord-length) splits every field
    record; the library's bytes equal numpy's and read back in either order."""
    sc = scenario(37, 18, 9, seed=62)
    shape = (sc.im, sc.jm, sc.km)
    gpu = _stepped(sc, 2)
    monkeypatch.setenv("LES_IO_MAX_SUBRECORD", "1001")
    p30, p31 = str(tmp_path / "r30"), str(tmp_path / "r31")
    gpu.write_data30(p30, 2, 0.05, big_endian=False)
    gpu.write_data31(p31)
    want30, want31 = _interiors(gpu, ftnio.DATA30, shape), _interiors(gpu, ftnio.DATA31, shape)
    for p, want, names, head, be in ((p30, want30, ftnio.DATA30, (2, 0.05), False),
                                     (p31, want31, ftnio.DATA31, None, True)):
        q = p + ".np"
        ftnio.write_fields(q, want, names, be, header=head, max_subrecord=1001)
        assert open(p, "rb").read() == open(q, "rb").read(), p
    other = make_gpu(scenario(37, 18, 9, seed=63), lesgpu.Params())
    n, t = other.read_restart(p30, p31)
    assert (n, np.float32(t)) == (2, np.float32(0.05))
    for nm, fid in IDS.items():
        _same(other.download(fid, (1, 1, 1), shape), gpu.download(fid, (1, 1, 1), shape), nm)


def test_ifdata_out_writes_at_n1_minus_1_and_nmax(built_lib, tmp_path):
    sc = scenario(32, 16, 8, seed=64)
    gpu = make_gpu(sc, lesgpu.Params())
    n1, nmax, dt = 3, 5, np.float32(0.05)
    wrote = []
    for n in range(1, nmax + 1):
        gpu.step(n, nmax)
        if gpu.ifdata_out(str(tmp_path), n, n1, nmax, float(np.float32(n - 1) * dt)):
            wrote.append(n)
    assert wrote == [n1 - 1, nmax]
    assert sorted(os.listdir(tmp_path)) == sorted(
        [ftnio.data30_name(2), ftnio.data31_name(2), ftnio.data30_name(5), ftnio.data31_name(5)])
    _, n, t = ftnio.read_fields(str(tmp_path / ftnio.data30_name(5)), ftnio.DATA30, (32, 16, 8), header=True)
    assert (n, np.float32(t)) == (5, np.float32(4) * dt)


def test_restart_continues_like_the_reference(built_lib, tmp_path):
    """ifdata's restart restores interiors only; the halos of a fresh set-up stay.  A
    restarted run equals a fresh domain given the same interiors (bit for bit) and
    the oracle doing the same (FP32 tolerance), and starts from the writer's state."""
    sc = scenario(48, 32, 16, seed=65)
    shape = (sc.im, sc.jm, sc.km)
    params = lesgpu.Params(nmaxp=20)
    nmax, nstop = 8, 4
    a = make_gpu(sc, params)
    for n in range(1, nstop + 1):
        a.step(n, nmax)
        a.ifdata_out(str(tmp_path), n, nstop + 1, nmax, float(np.float32(n - 1) * np.float32(0.05)))
    p30, p31 = str(tmp_path / ftnio.data30_name(nstop)), str(tmp_path / ftnio.data31_name(nstop))

    b = make_gpu(sc, params)
    n0, _ = b.read_restart(p30, p31)
    assert n0 == nstop
    for nm, fid in IDS.items():
        _same(b.download(fid, (1, 1, 1), shape), a.download(fid, (1, 1, 1), shape), ("loaded", nm))

    f30, _, _ = ftnio.read_fields(p30, ftnio.DATA30, shape, header=True)
    f31, _, _ = ftnio.read_fields(p31, ftnio.DATA31, shape)
    state = {**f30, **f31}
    c = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    for nm, arr in state.items():
        c.upload(IDS[nm], arr, (1, 1, 1), shape)
        orc.set(IDS[nm], arr, (1, 1, 1), shape)
    for n in range(nstop + 1, nmax + 1):
        b.step(n, nmax)
        c.step(n, nmax)
        orc.step(n, nmax)
    for nm, fid in IDS.items():
        _same(b.download(fid), c.download(fid), ("restarted", nm))
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P):
        e = rel_err(b.download(fid, (1, 1, 1), shape).astype(np.float64), orc.get(fid, (1, 1, 1), shape))
        assert e <= 1e-5, (lesgpu.FIELD_NAMES[fid], e)


def test_bad_files_fail_with_a_message(built_lib, tmp_path):
    sc = scenario(24, 12, 6, seed=66)
    gpu = make_gpu(sc, lesgpu.Params())
    small = make_gpu(scenario(20, 12, 6, seed=66), lesgpu.Params())
    p30, p31 = str(tmp_path / "s30"), str(tmp_path / "s31")
    small.write_data30(p30, 1, 0.0)
    small.write_data31(p31)
    with pytest.raises(lesgpu.LesError, match="fewer values"):
        gpu.read_restart(p30, p31)
    with pytest.raises(lesgpu.LesError, match="cannot open"):
        gpu.read_restart(str(tmp_path / "missing"), p31)
    (tmp_path / "junk").write_bytes(b"\x00\x00\x00\x09not a record")
    with pytest.raises(lesgpu.LesError, match="record markers"):
        gpu.read_restart(str(tmp_path / "junk"), p31)
    with pytest.raises(lesgpu.LesError, match="cannot open"):
        gpu.write_data20(str(tmp_path / "no" / "such" / "dir" / "data20"))


def test_longer_records_are_read_like_fortran(built_lib, tmp_path):
    """A Fortran read of fewer values than the record holds takes the first ones and
    moves on to the next record (ifdata.f95:252-480 reads im*jm*km values per record):
    records with trailing extra values, written by the independent writer, load the same
    interiors as exact ones."""
    import struct
    sc = scenario(20, 12, 6, seed=67)
    shape = (sc.im, sc.jm, sc.km)
    rng = np.random.default_rng(68)
    f30 = {nm: rng.standard_normal(shape).astype(np.float32) for nm in ftnio.DATA30}
    f31 = {nm: rng.standard_normal(shape).astype(np.float32) for nm in ftnio.DATA31}
    tail = np.arange(5, dtype=np.float32)
    p30, p31 = str(tmp_path / "long30"), str(tmp_path / "long31")
    ftnio.write_records(p30, [struct.pack(">if", 9, 0.4) + b"\0" * 8] +
                        [np.concatenate([f30[nm].ravel(order="F"), tail]) for nm in ftnio.DATA30])
    ftnio.write_records(p31, [np.concatenate([f31[nm].ravel(order="F"), tail]) for nm in ftnio.DATA31])
    gpu = make_gpu(sc, lesgpu.Params())
    n, t = gpu.read_restart(p30, p31)
    assert (n, np.float32(t)) == (9, np.float32(0.4))
    for nm, arr in {**f30, **f31}.items():
        _same(gpu.download(IDS[nm], (1, 1, 1), shape), arr, nm)
