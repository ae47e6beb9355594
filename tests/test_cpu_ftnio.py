"""CPU checks of the reference's unformatted file format (ftnio): record markers, byte
order, subrecords and the data20/data30/data31 layouts, against byte strings built
by hand from gfortran's documented layout."""
import struct

import numpy as np
import pytest

import ftnio


def _be(v):
    return struct.pack(">i", v)


def _le(v):
    return struct.pack("<i", v)


def test_header_record_bytes(tmp_path):
    """write(30) n,time with -fconvert=big-endian: marker 8, int32 n, real(4) time, 8."""
    p = tmp_path / "h.dat"
    ftnio.write_records(str(p), [struct.pack(">if", 48000, 2400.0)])
    assert p.read_bytes() == _be(8) + _be(48000) + struct.pack(">f", 2400.0) + _be(8)
    ftnio.write_records(str(p), [struct.pack("<if", 48000, 2400.0)], big_endian=False)
    assert p.read_bytes() == _le(8) + _le(48000) + struct.pack("<f", 2400.0) + _le(8)


def test_field_record_is_i_fastest_big_endian(tmp_path):
    """(((u(i,j,k),i=1,im),j=1,jm),k=1,km): i varies fastest."""
    im, jm, km = 3, 2, 2
    u = np.zeros((im, jm, km), np.float32, order="F")
    for i in range(im):
        for j in range(jm):
            for k in range(km):
                u[i, j, k] = 100 * (i + 1) + 10 * (j + 1) + (k + 1)
    p = tmp_path / "u.dat"
    ftnio.write_records(str(p), [u])
    want = [100 * i + 10 * j + k for k in (1, 2) for j in (1, 2) for i in (1, 2, 3)]
    body = b"".join(struct.pack(">f", float(x)) for x in want)
    assert p.read_bytes() == _be(48) + body + _be(48)


def test_subrecord_split(tmp_path):
    """A 24-byte record with at most 10 bytes per subrecord: 10, 10, 4; leading markers
    negative while another follows, trailing markers negative after the first."""
    data = bytes(range(24))
    p = tmp_path / "s.dat"
    ftnio.write_records(str(p), [data, b"xy"], max_subrecord=10)
    want = (_be(-10) + data[0:10] + _be(10) + _be(-10) + data[10:20] + _be(-10) + _be(4) + data[20:] + _be(-4)
            + _be(2) + b"xy" + _be(2))
    assert p.read_bytes() == want
    recs, be = ftnio.read_records(str(p))
    assert be and recs == [data, b"xy"]


def test_split_inside_a_value(tmp_path):
    """Subrecords split on bytes, not values: a 6-byte limit cuts floats in half."""
    a = np.arange(1, 8, dtype=np.float32).reshape(7, 1, 1, order="F")
    p = tmp_path / "c.dat"
    ftnio.write_fields(str(p), {"u": a}, ["u"], max_subrecord=6)
    got, _, _ = ftnio.read_fields(str(p), ["u"], a.shape)
    assert np.array_equal(got["u"], a)


@pytest.mark.parametrize("big_endian", [True, False])
def test_data30_data31_round_trip(tmp_path, big_endian):
    rng = np.random.default_rng(5)
    shape = (7, 5, 4)
    f30 = {nm: rng.standard_normal(shape).astype(np.float32) for nm in ftnio.DATA30}
    f31 = {nm: rng.standard_normal(shape).astype(np.float32) for nm in ftnio.DATA31}
    p30, p31 = tmp_path / ftnio.data30_name(120), tmp_path / ftnio.data31_name(120)
    ftnio.write_fields(str(p30), f30, ftnio.DATA30, big_endian, header=(120, 6.25))
    ftnio.write_fields(str(p31), f31, ftnio.DATA31, big_endian)
    assert ftnio.detect_order(str(p30)) is big_endian
    got30, n, t = ftnio.read_fields(str(p30), ftnio.DATA30, shape, header=True)
    got31, _, _ = ftnio.read_fields(str(p31), ftnio.DATA31, shape)
    assert (n, t) == (120, 6.25)
    for nm in ftnio.DATA30:
        assert np.array_equal(got30[nm].view(np.uint32), f30[nm].view(np.uint32)), nm
    for nm in ftnio.DATA31:
        assert np.array_equal(got31[nm].view(np.uint32), f31[nm].view(np.uint32)), nm
    # 8-byte header record, then 7 records of im*jm*km values, each with two markers
    n3 = 4 * shape[0] * shape[1] * shape[2]
    assert p30.stat().st_size == 16 + 7 * (n3 + 8)
    assert p31.stat().st_size == 6 * (n3 + 8)


def test_file_names_follow_i6_6():
    """anime.f95:375 and :492 name files with i6.6; ifdata.f95:257 opens data30048000.dat."""
    assert ftnio.data30_name(48000) == "data30048000.dat"
    assert ftnio.data31_name(7) == "data31000007.dat"


def test_reading_fewer_values_than_the_record_holds(tmp_path):
    """A Fortran read of fewer values than the record holds takes the first ones."""
    p = tmp_path / "l.dat"
    a = np.arange(30, dtype=np.float32)
    ftnio.write_records(str(p), [a])
    got, _, _ = ftnio.read_fields(str(p), ["x"], (2, 3, 4))
    assert np.array_equal(got["x"].ravel(order="F"), a[:24])
    with pytest.raises(ValueError):
        ftnio.read_fields(str(p), ["x"], (4, 4, 2))


def test_bad_markers_are_refused(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_bytes(_be(8) + b"12345678" + _be(7))
    with pytest.raises(ValueError):
        ftnio.read_records(str(p))
    p.write_bytes(_be(8) + b"1234")
    with pytest.raises(ValueError):
        ftnio.detect_order(str(p))


def test_compare_two_runs_files(tmp_path):
    """ftnio.compare: per-field differences of two files of one kind, in either byte
    order (a GPU run's data20 against a reference run's)."""
    rng = np.random.default_rng(8)
    shape = (6, 5, 4)
    a = {nm: rng.standard_normal(shape).astype(np.float32) for nm in ftnio.DATA20}
    b = {nm: v.copy() for nm, v in a.items()}
    b["p"][2, 3, 1] += np.float32(0.5)
    b["w"][0, 0, 0] = np.nan
    pa, pb = tmp_path / "data20", tmp_path / "data20.le"
    ftnio.write_fields(str(pa), a, ftnio.DATA20)
    ftnio.write_fields(str(pb), b, ftnio.DATA20, big_endian=False)
    d = ftnio.compare(str(pa), str(pb), shape, kind="data20")
    assert d["u"] == (0.0, 0.0)
    assert abs(d["p"][0] - 0.5) < 1e-6 and d["p"][1] > 0
    assert d["w"][0] == np.inf
    assert ftnio.kind_of(str(tmp_path / ftnio.data30_name(5))) == "data30"
    assert ftnio.main([str(pa), "--dims", "6x5x4"]) == 0
    assert ftnio.main([str(pa), str(pb), "--dims", "6x5x4"]) == 0
