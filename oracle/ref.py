"""ctypes binding of the CPU oracle (oracle/les_ref.cpp).

TEST INFRASTRUCTURE ONLY: the parity checker.  Only the tests, the smoke check and
the benchmark's CPU-baseline leg use it; the GPU product never imports it.

``Ref`` holds one domain in the oracle (FP32 = the reference's real(kind=4), or FP64
= the reference built with -freal-4-real-8) and runs the reference's subroutines
stage by stage.  Fields cross in the reference's Fortran layout (numpy, order='F').
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

STEP, VELNW, BONDV1, VELFG, FEEDBF, LES, ADAM, PRESS, BOUNDP1, BOUNDP2, BONDFG = range(11)

_libs: dict[str, C.CDLL] = {}


def build() -> None:
    """Compile the oracle libraries (make in oracle/)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load(fast: bool = False) -> C.CDLL:
    name = "liblesref_fast.so" if fast else "liblesref.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        build()
    lib = C.CDLL(path)
    vp, dp, ip_ = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    fp_ = C.POINTER(C.c_float)
    lib.ref_create.restype = vp
    lib.ref_create.argtypes = [C.c_int] * 4 + [dp, ip_, fp_, fp_, fp_, fp_]
    lib.ref_destroy.argtypes = [vp]
    lib.ref_stage.restype = C.c_int
    lib.ref_stage.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    lib.ref_aveflow.restype = C.c_int
    lib.ref_aveflow.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    for n in ("ref_get", "ref_set"):
        getattr(lib, n).restype = C.c_int
        getattr(lib, n).argtypes = [vp, C.c_int, dp, ip_, ip_]
    lib.ref_extents.restype = C.c_int
    lib.ref_extents.argtypes = [vp, C.c_int, ip_, ip_]
    lib.ref_diag.argtypes = [vp, dp]
    lib.ref_bounds_checked.restype = C.c_int
    lib.ref_last_error.restype = C.c_char_p
    lib.ref_set_threads.restype = C.c_int
    lib.ref_set_threads.argtypes = [C.c_int]
    lib.ref_trap_wall.restype = C.c_int
    lib.ref_trap_wall.argtypes = [vp, C.c_int]
    lib.ref_scenario.restype = C.c_int
    lib.ref_scenario.argtypes = [C.c_int] * 3 + [fp_, ip_, C.c_ulonglong, fp_, fp_, fp_, fp_]
    _libs[name] = lib
    return lib


def set_threads(n: int, fast: bool = True) -> int:
    """Threads of the fast build's parallel loops (OMP_NUM_THREADS is read once, when
    the OpenMP runtime starts -- often at `import torch` -- so it cannot be relied on);
    returns the count the next steps use."""
    return int(load(fast).ref_set_threads(int(n)))


def scenario(im: int, jm: int, km: int, seed: int = 1, *, dz_law: int = 1, dz0: float = 2.0,
             dz_ratio: float = 1.04, coverage: float = 0.30, fp_min: int = 5, fp_max: int = 20,
             h_min: float = 10.0, h_max: float = 60.0, inflow_law: int = 1, u_ref: float = 5.0,
             z_ref: float = 100.0, pl_exp: float = 0.2, direction_deg: float = 0.0, noise: float = 1e-3,
             fast: bool = False, **_ignored):
    """The configs' seeded synthetic scenario as the oracle restates it: (zbm[im,jm],
    uin[jm,km], vin, win), Fortran-ordered float32.  The defaults are the workload's
    (30 % coverage of 5-20-cell blocks 10-60 m high, 5 m/s (z/100 m)^0.2 inflow with
    +-1e-3 m/s noise, dz = 2 m x 1.04)."""
    lib = load(fast)
    fl = np.array([dz0, dz_ratio, coverage, h_min, h_max, u_ref, z_ref, pl_exp, direction_deg, noise], np.float32)
    iv = np.array([dz_law, fp_min, fp_max, inflow_law], np.int32)
    zbm = np.zeros((im, jm), np.float32, order="F")
    uin, vin, win = (np.zeros((jm, km), np.float32, order="F") for _ in range(3))
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rc = lib.ref_scenario(im, jm, km, f(fl), iv.ctypes.data_as(C.POINTER(C.c_int)), C.c_ulonglong(seed), f(zbm),
                          f(uin), f(vin), f(win))
    if rc:
        raise RuntimeError("ref_scenario: " + lib.ref_last_error().decode())
    return zbm, uin, vin, win


class Ref:
    """One domain in the oracle.  prec 4 (FP32) or 8 (FP64)."""

    def __init__(self, prec: int, im: int, jm: int, km: int, zbm, uin, vin, win, *, dt=0.05, ro=1.1763,
                 vn=None, alpha=-10.0, beta=-1.0, omega=1.0, pjuge=1e-4, dx=4.0, dy=4.0, dz_law=1, dz0=2.0,
                 dz_ratio=1.04, nmaxp=50, sor_fixed=1, red64=1, sqrt_half=1, fast=False):
        self.lib = load(fast)
        self.im, self.jm, self.km, self.prec = im, jm, km, prec
        if vn is None:
            vn = float(np.float32(15.83) * np.float32(1e-6)) if prec == 4 else 15.83e-6
        consts = (C.c_double * 11)(dt, ro, vn, alpha, beta, omega, pjuge, dx, dy, dz0, dz_ratio)
        opts = (C.c_int * 5)(nmaxp, sor_fixed, red64, sqrt_half, dz_law)
        self._keep = [np.asfortranarray(x, dtype=np.float32) for x in (zbm, uin, vin, win)]
        ptrs = [x.ctypes.data_as(C.POINTER(C.c_float)) for x in self._keep]
        self._h = self.lib.ref_create(prec, im, jm, km, consts, opts, *ptrs)
        if not self._h:
            raise RuntimeError("ref_create: " + self.lib.ref_last_error().decode())

    def close(self):
        if self._h:
            self.lib.ref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stage(self, s: int, n: int = 1, nmax: int = 1):
        rc = self.lib.ref_stage(self._h, s, n, nmax)
        if rc:
            raise RuntimeError(f"ref_stage({s}): " + self.lib.ref_last_error().decode())

    def step(self, n: int, nmax: int):
        self.stage(STEP, n, nmax)

    def trap_wall(self, on: bool = True):
        """Stop velfg with an error where a wall speed is zero (vel2.f95:138,173: the
        reference forms 0/0 there) instead of carrying on with the NaN."""
        self.lib.ref_trap_wall(self._h, 1 if on else 0)

    def aveflow(self, n: int, n1: int, nmax: int):
        """aveflow.f95: accumulate the time averages at step n (from n1), finalise at nmax."""
        if self.lib.ref_aveflow(self._h, n, n1, nmax):
            raise RuntimeError("ref_aveflow: " + self.lib.ref_last_error().decode())

    def extents(self, fid: int):
        lb, ub = (C.c_int * 3)(), (C.c_int * 3)()
        if self.lib.ref_extents(self._h, fid, lb, ub):
            raise KeyError(fid)
        return tuple(lb), tuple(ub)

    def get(self, fid: int, lb=None, ub=None) -> np.ndarray:
        dlb, dub = self.extents(fid)
        lb = tuple(lb) if lb is not None else dlb
        ub = tuple(ub) if ub is not None else dub
        shape = tuple(ub[q] - lb[q] + 1 for q in range(3))
        out = np.zeros(shape, np.float64, order="F")
        rc = self.lib.ref_get(self._h, fid, out.ctypes.data_as(C.POINTER(C.c_double)), (C.c_int * 3)(*lb),
                              (C.c_int * 3)(*ub))
        if rc:
            raise RuntimeError(f"ref_get({fid}): " + self.lib.ref_last_error().decode())
        return out

    def set(self, fid: int, arr, lb=None, ub=None):
        dlb, dub = self.extents(fid)
        lb = tuple(lb) if lb is not None else dlb
        ub = tuple(ub) if ub is not None else dub
        a = np.asfortranarray(arr, dtype=np.float64)
        rc = self.lib.ref_set(self._h, fid, a.ctypes.data_as(C.POINTER(C.c_double)), (C.c_int * 3)(*lb),
                              (C.c_int * 3)(*ub))
        if rc:
            raise RuntimeError(f"ref_set({fid}): " + self.lib.ref_last_error().decode())

    def diag(self) -> dict:
        out = (C.c_double * 7)()
        self.lib.ref_diag(self._h, out)
        return {"iters": int(out[0]), "sor": out[1], "uout": out[2], "rhsav": out[3], "pav": out[4],
                "area": out[5], "pco": out[6]}
