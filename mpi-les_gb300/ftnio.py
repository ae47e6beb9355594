"""Read and write the reference's unformatted result and restart files with numpy.

The reference writes its results and restart state as gfortran unformatted
sequential files, big-endian (``-fconvert=big-endian``, SConstruct:77):

==================  ==========================  =============================================
file                written by                  records
==================  ==========================  =============================================
data20              press.f95:205-216           u, v, w, p, usum, vsum, wsum
data21              adam.f95:20-27              fold, gold, hold, fghold
data30NNNNNN.dat    anime.f95:370-490           (n, time), u, v, w, p, usum, vsum, wsum
data31NNNNNN.dat    anime.f95:492-595           f, g, h, fold, gold, hold
data10              aveflow.f95:209-263         aveu, avew, avev
data11              aveflow.f95:273-344         aveuu, aveww, avevv, uwfx
==================  ==========================  =============================================

Every 3-D record is the box (1:im, 1:jm, 1:km) with i fastest: here a
Fortran-ordered float32 array of shape (im, jm, km).  The GPU library writes and
reads the same files from device state (``Domain.write_data20`` ...,
``Domain.read_restart``); this module reads them on any host, writes them from
numpy arrays, and serves as the independent second implementation the library's
files are checked against.

Record layout (gfortran's documented format): a record is one or more
subrecords, each a 4-byte length marker, the data and the marker again.  A
subrecord holds at most 2147483639 bytes; a longer record is split, the leading
marker of every subrecord but the last negated and the trailing marker of every
subrecord but the first negated.
"""
from __future__ import annotations

import os
import struct

import numpy as np

MAX_SUBRECORD = 2147483639

DATA20 = ("u", "v", "w", "p", "usum", "vsum", "wsum")
DATA21 = ("fold", "gold", "hold", "fghold")
DATA30 = DATA20
DATA31 = ("f", "g", "h", "fold", "gold", "hold")
DATA10 = ("aveu", "avew", "avev")
DATA11 = ("aveuu", "aveww", "avevv", "uwfx")


def write_records(path: str, records, big_endian: bool = True, max_subrecord: int = MAX_SUBRECORD) -> None:
    """Write each item of `records` (bytes, or a numpy array written as its
    Fortran-order values in the file's byte order) as one record."""
    if not 1 <= max_subrecord <= MAX_SUBRECORD:
        raise ValueError("max_subrecord out of range")
    mk = ">i4" if big_endian else "<i4"
    with open(path, "wb") as f:
        for rec in records:
            if isinstance(rec, np.ndarray):
                dt = rec.dtype.newbyteorder(">" if big_endian else "<")
                data = np.asarray(rec, order="F").astype(dt).tobytes(order="F")
            else:
                data = bytes(rec)
            off, first = 0, True
            while True:
                ln = min(len(data) - off, max_subrecord)
                last = off + ln == len(data)
                f.write(np.array([ln if last else -ln], mk).tobytes())
                f.write(data[off:off + ln])
                f.write(np.array([ln if first else -ln], mk).tobytes())
                off += ln
                first = False
                if off >= len(data):
                    break


def detect_order(path: str) -> bool:
    """True for a big-endian file, False for little-endian, from the first record's
    markers (big-endian is tried first); ValueError if neither order fits."""
    size = os.path.getsize(path)
    with open(path, "rb") as f:
        lead = f.read(4)
        if size < 8 or len(lead) < 4:
            raise ValueError(f"{path}: too short for a Fortran record")
        for be in (True, False):
            (v,) = struct.unpack(">i" if be else "<i", lead)
            ln = abs(v)
            if 8 + ln > size:
                continue
            f.seek(4 + ln)
            (t,) = struct.unpack(">i" if be else "<i", f.read(4))
            if t == ln:
                return be
    raise ValueError(f"{path}: not a Fortran unformatted sequential file (record markers do not match)")


def read_records(path: str, big_endian: bool | None = None) -> tuple[list[bytes], bool]:
    """Every record of the file as raw bytes (subrecords joined), and the byte order."""
    be = detect_order(path) if big_endian is None else big_endian
    fmt = ">i" if be else "<i"
    out = []
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if not head:
                break
            parts, first = [], True
            while True:
                if len(head) < 4:
                    raise ValueError(f"{path}: record {len(out) + 1}: ends inside a marker")
                (lead,) = struct.unpack(fmt, head)
                data = f.read(abs(lead))
                tail = f.read(4)
                if len(data) < abs(lead) or len(tail) < 4:
                    raise ValueError(f"{path}: record {len(out) + 1}: cut short")
                (trail,) = struct.unpack(fmt, tail)
                if abs(trail) != abs(lead) or (trail < 0) == first:
                    raise ValueError(f"{path}: record {len(out) + 1}: leading and trailing markers disagree")
                parts.append(data)
                if lead >= 0:
                    break
                head, first = f.read(4), False
            out.append(b"".join(parts))
    return out, be


def _field(rec: bytes, shape, be: bool, path: str, name: str) -> np.ndarray:
    n = shape[0] * shape[1] * shape[2]
    if len(rec) < 4 * n:
        raise ValueError(f"{path}: record {name} holds {len(rec) // 4} values, {n} expected")
    a = np.frombuffer(rec[:4 * n], dtype=">f4" if be else "<f4").astype(np.float32)
    return a.reshape(shape, order="F")


def read_fields(path: str, names, shape, header: bool = False):
    """Read a file of 3-D records named `names` (each of `shape` = (im, jm, km));
    with header=True the first record is (n, time).  Returns ({name: array}, n, time)."""
    recs, be = read_records(path)
    need = len(names) + (1 if header else 0)
    if len(recs) < need:
        raise ValueError(f"{path}: {len(recs)} records, {need} expected")
    n = t = None
    if header:
        if len(recs[0]) < 8:
            raise ValueError(f"{path}: first record shorter than (n, time)")
        n, t = struct.unpack(">if" if be else "<if", recs[0][:8])
        recs = recs[1:]
    return {nm: _field(r, shape, be, path, nm) for nm, r in zip(names, recs)}, n, t


def write_fields(path: str, fields: dict, names, big_endian: bool = True, header=None,
                 max_subrecord: int = MAX_SUBRECORD) -> None:
    """Write the named arrays (float32, shape (im, jm, km)) as one record each, after
    an (n, time) record when header = (n, time)."""
    recs = []
    if header is not None:
        recs.append(struct.pack(">if" if big_endian else "<if", int(header[0]), float(header[1])))
    recs += [np.asarray(fields[nm], np.float32) for nm in names]
    write_records(path, recs, big_endian, max_subrecord)


def data30_name(n: int) -> str:
    """anime.f95:375: '("data30",i6.6,".dat")'."""
    return f"data30{n:06d}.dat"


def data31_name(n: int) -> str:
    """anime.f95:492: '("data31",i6.6,".dat")'."""
    return f"data31{n:06d}.dat"


LAYOUTS = {  # file kind -> (record names, leading (n, time) record)
    "data20": (DATA20, False), "data21": (DATA21, False), "data30": (DATA30, True), "data31": (DATA31, False),
    "data10": (DATA10, False), "data11": (DATA11, False),
}


def kind_of(path: str) -> str:
    """The file kind from the reference's naming (data20, data30NNNNNN.dat, ...)."""
    base = os.path.basename(path)
    for k in LAYOUTS:
        if base.startswith(k):
            return k
    raise ValueError(f"{path}: not one of the reference's file names ({', '.join(LAYOUTS)})")


def compare(path_a: str, path_b: str, shape, kind: str | None = None) -> dict:
    """Per-field differences of two files of one kind (a GPU run against a reference
    run, two restarts, ...): {name: (max |a-b|, max |a-b| / max |b|)}, NaNs counted
    as differences unless both sides hold them.  The files may differ in byte order."""
    kind = kind or kind_of(path_a)
    names, header = LAYOUTS[kind]
    fa, na, ta = read_fields(path_a, names, shape, header=header)
    fb, nb, tb = read_fields(path_b, names, shape, header=header)
    out = {}
    if header:
        out["(n, time)"] = (float(abs(na - nb)), float(abs(np.float32(ta) - np.float32(tb))))
    for nm in names:
        a, b = fa[nm].astype(np.float64), fb[nm].astype(np.float64)
        both_nan = np.isnan(a) & np.isnan(b)
        d = np.where(both_nan, 0.0, np.abs(a - b))
        d = np.where(np.isnan(d), np.inf, d)
        scale = float(np.nanmax(np.abs(b))) if np.isfinite(b).any() else 0.0
        dmax = float(d.max()) if d.size else 0.0
        out[nm] = (dmax, dmax / scale if scale > 0 else (0.0 if dmax == 0 else np.inf))
    return out


def main(argv=None) -> int:
    """python ftnio.py FILE [FILE2] --dims IMxJMxKM: list the records of a reference file
    (per field min, max, mean) or compare two (per field max abs and relative difference)."""
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("files", nargs="+")
    ap.add_argument("--dims", required=True, help="IMxJMxKM of the domain the file holds")
    args = ap.parse_args(argv)
    shape = tuple(int(x) for x in args.dims.split("x"))
    if len(args.files) == 2:
        for nm, (dabs, drel) in compare(args.files[0], args.files[1], shape).items():
            print(f"{nm:10s} max |a-b| {dabs:.6g}   relative {drel:.3g}")
        return 0
    path = args.files[0]
    names, header = LAYOUTS[kind_of(path)]
    fields, n, t = read_fields(path, names, shape, header=header)
    print(f"{path}: {'big' if detect_order(path) else 'little'}-endian" + (f", n = {n}, time = {t:g}" if header else ""))
    for nm in names:
        a = fields[nm]
        print(f"{nm:10s} min {np.nanmin(a):.6g}  max {np.nanmax(a):.6g}  mean {np.nanmean(a):.6g}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
